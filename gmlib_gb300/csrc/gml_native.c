/*
 * gml_native.c -- host side of the native mesh kernels (no counterpart in the
 * reference API).  Filled in by the native smoothing / quality extensions.
 */
#include <stdlib.h>
#include "gml_internal.h"
#include "gmlib3_gb300.h"

void gmlx_native_release(GmlSct *gml)
{
   (void)gml;
}
