// Device-only translation unit holding the reference's own traversal kernels,
// trace_kernel and trace_shadow_kernel (src/renderer/pathtracer_kernel.h:175-321),
// compiled from the reference sources where they lie by build_ref.sh into
// cubins under oracle/_ref/. oracle/ref_gpu.py loads them through the CUDA
// driver API and launches them as the reference's trace() / trace_shadow()
// wrappers do (32-thread blocks, pathtracer_kernel.h:235-246, 310-321).
// Test and bench infrastructure: the product never loads them.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <device_launch_parameters.h>
#include "renderer/pathtracer_kernel.h"
