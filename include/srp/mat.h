/* srp-gb300 public API: 4x4 row-major matrices.
 *
 * Replaces include/srp/mat.h of kitrofimov/srp (mat.h:16-93). Products are
 * evaluated left to right in plain fp32 (no FMA), which is what makes vertex
 * positions, and therefore coverage and depth, bit-identical to the reference.
 * The constructors that take angles use double sin/cos on the host. */
#pragma once

#include "srp/vec.h"

#if defined(__cplusplus)
#define SRP_RESTRICT __restrict__
#else
#define SRP_RESTRICT restrict
#endif

typedef struct mat4 { float data[4][4]; } mat4;

#ifdef __cplusplus
extern "C" {
#endif

vec4 mat4MultiplyVec4(const mat4* SRP_RESTRICT a, vec4 b);                          /* mat.h:22 */
mat4 mat4MultiplyMat4(const mat4* SRP_RESTRICT a, const mat4* SRP_RESTRICT b);      /* mat.h:28 */
mat4 mat4ConstructIdentity(void);                                                   /* mat.h:32 */
mat4 mat4ConstructScale(float x, float y, float z);                                 /* mat.h:37 */
mat4 mat4ConstructTranslate(float x, float y, float z);                             /* mat.h:41 */
mat4 mat4ConstructRotate(float x, float y, float z);                                /* mat.h:46 */
mat4 mat4ConstructTRS(float transX, float transY, float transZ,
                      float rotationX, float rotationY, float rotationZ,
                      float scaleX, float scaleY, float scaleZ);                    /* mat.h:52-56 */
mat4 mat4ConstructView(float cameraX, float cameraY, float cameraZ,
                       float rotationX, float rotationY, float rotationZ,
                       float scaleX, float scaleY, float scaleZ);                   /* mat.h:63-67 */
mat4 mat4ConstructOrthogonalProjection(float x_min, float x_max, float y_min, float y_max,
                                       float z_min, float z_max);                   /* mat.h:76-80 */
mat4 mat4ConstructPerspectiveProjection(float x_min_near, float x_max_near,
                                        float y_min_near, float y_max_near,
                                        float z_near, float z_far);                 /* mat.h:89-93 */

#ifdef __cplusplus
}
#endif
