// Stand-in for Common/Scenes/Model.h with only what Model::Scale
// (Model.cpp:647-710) touches: the vertex array and its length.  The real
// header pulls in every acceleration structure and Direct3D; build_ref.sh
// compiles the reference's own Model::Scale body against this declaration.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include "Vertex.h"

using std::max;

class Model {
public:
    Vertex* m_pVertices = nullptr;
    unsigned int m_uiNumVertices = 0;
    void Scale();
};
