/*
 * Test infrastructure: force-included (-include) when compiling an unmodified
 * Object-MD application against the GPU integrator.  The reference's headers
 * come in first, then the drop-in; from there on the application's own text
 * reads GPUIntegrator wherever it names MDIntegrator, which is the one-line
 * swap objectmd_gb300/dropin/gpu_integrator.h describes.
 */
#include <omd.h>
#include "gpu_integrator.h"
#define MDIntegrator GPUIntegrator
