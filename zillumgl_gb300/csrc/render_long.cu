// render_long.cu — the integrator kernels of render_kernels.cuh with long
// rays finished by the lanes that trace together (shading.cuh: a ray with a
// near-zero direction component that outruns kLongRayBudget table entries is
// walked by its lane group, 32 entries per window).  The integrator entry
// points (render.cu) launch these for trees of at least kLongRayMinEntries
// entries.
#define ZGL_LONG_RAYS 1
#define ZGL_RENDER_NS long_rays
#include "render_kernels.cuh"
