/* Host build of the shared shader library for programs linked against the
 * CPU oracle or the reference library (the GPU library exports its own). */
#include "srp/shaderlib_host.inc"
