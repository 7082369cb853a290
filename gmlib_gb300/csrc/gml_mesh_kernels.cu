/*
 * gml_mesh_kernels.cu -- native mesh kernels (quality, smoothing, topology
 * builders) with no counterpart in the reference API.
 */
#include <cuda_runtime.h>
#include "gml_device.h"
