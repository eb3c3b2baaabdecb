// mpf3d_internal.h -- shared definitions of the libmpf3d translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define MPF3D_VERSION 1
