// The fast build of the ray caster's march (namespace gc::fast): the same
// source as render.cu compiled with FMA contraction, rsqrtf in normalize, the
// hardware log2/exp2 pair for the opacity correction and multiplies by
// reciprocals for the voxel normalisation -- the operations the reference's
// own build uses (nvcc defaults, RayCasters.cu).  Selected with
// gc_render_precision_set(GC_RENDER_FAST_BUILD); its images are compared with
// the double-precision oracle and the reference's ray caster, not with the
// FP32 oracle bit for bit.
#define GC_RENDER_FAST 1
#include "render.cu"
