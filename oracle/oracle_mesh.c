/*
 * oracle_mesh.c -- CPU restatement of the native mesh kernels (Laplacian
 * smoothing over the ball of points, mean-ratio quality histogram, inverted
 * element flags) and of the block sparse solvers.  TEST INFRASTRUCTURE ONLY.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"
