/*
 * rt_model.h -- headless model ingestion for the LBVH core (librthost.so).
 *
 * Replaces Model::LoadFile and Model::Scale (Common/Scenes/Model.cpp:107-113,
 * 210-381, 647-709) without the Direct3D material / texture objects: a model
 * file becomes the fp32 triangle soup (n x 9 floats: A.xyz B.xyz C.xyz) that
 * rt_lbvh_build takes, plus a material id per triangle and the materials'
 * colours.
 *
 *  .obj  Wavefront OBJ as the reference's loader reads it
 *        (Common/Scenes/Loaders/model_obj.cpp): v / vt / vn records, faces in
 *        the forms v, v/vt, v//vn and v/vt/vn, polygons split into the fan
 *        (v0, v_k, v_k+1), negative indices resolved as that loader does
 *        (-k -> count - k - 1, one below the OBJ convention), usemtl / mtllib
 *        (newmtl, Ka, Kd, Ks, Ns, d, Tr), then normalize(): centred on the
 *        bounds' centre and scaled by 1 / (largest extent).
 *  .txt  the reference's text format: vertex count, triangle count, the
 *        vertices (position, normal, u, v), then three indices per triangle.
 *
 * Both then get Model::Scale: into the box of half-size 0.9 about the origin,
 * then into the sphere of radius 0.49, over the model's vertices (for .obj
 * the vertices the faces use; for .txt every vertex of the file).
 */
#ifndef RT_MODEL_H
#define RT_MODEL_H

#include <stddef.h>
#include <stdint.h>

#include "rt_api.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rt_model rt_model;

/* rt_material (include/rt_api.h): the MTL colours, Ns / 1000, and d or 1 - Tr. */

/* Loads `path` (.obj / .txt by extension, either case).  On failure returns
 * RT_ERR_INVALID and, when err is not NULL, a message in err[0 .. errlen). */
rt_status rt_model_load(const char* path, rt_model** out, char* err, size_t errlen);
void rt_model_free(rt_model* model);
uint32_t rt_model_triangle_count(const rt_model* model);
/* n x 9 floats, valid until rt_model_free. */
const float* rt_model_soup(const rt_model* model);
/* material id of each triangle (0 when the model has fewer than two). */
const int32_t* rt_model_material_ids(const rt_model* model);
uint32_t rt_model_material_count(const rt_model* model);
const rt_material* rt_model_material(const rt_model* model, uint32_t i);

#ifdef __cplusplus
}
#endif
#endif /* RT_MODEL_H */
