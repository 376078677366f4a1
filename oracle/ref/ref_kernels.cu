// Device-only translation unit holding the reference's own kernels
// (src/renderer/pathtracer_kernel.h: generate_primary_rays_kernel, trace_kernel,
// shade_hit_with_MIS_kernel, trace_shadow_kernel, the two accumulate kernels and
// finish_sample_kernel), compiled from the reference sources where they lie by
// build_ref.sh into cubins under oracle/_ref/. oracle/ref_gpu.py loads them
// through the CUDA driver API and launches them with the reference's launch
// shapes (its wrappers at pathtracer_kernel.h:106-117, 235-246, 310-321, 630-640,
// 666-682, 751-767, 782-790); oracle/ref_frame.cpp runs its frame loop.
// Test and bench infrastructure: the product never loads them.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <device_launch_parameters.h>
#include "renderer/pathtracer_kernel.h"
