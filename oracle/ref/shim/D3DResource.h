/* Minimal stand-in for the Direct3D resource header, used only when the
 * reference's CPU acceleration-structure sources are compiled as a test
 * oracle.  The CPU builders never touch GPU resources; they only need the
 * type names that Material.h / MaterialTextures.h mention. */
#ifndef RT_ORACLE_SHIM_D3DRESOURCE_H
#define RT_ORACLE_SHIM_D3DRESOURCE_H
#include <string>
struct ID3D11Device;
class D3DResource {};
#endif
