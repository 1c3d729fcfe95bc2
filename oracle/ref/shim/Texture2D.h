/* Empty stand-in: the texture class is a Direct3D type the CPU builders
 * never use. */
#ifndef RT_ORACLE_SHIM_TEXTURE2D_H
#define RT_ORACLE_SHIM_TEXTURE2D_H
#endif
