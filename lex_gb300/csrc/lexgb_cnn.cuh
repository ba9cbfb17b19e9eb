// lexgb_cnn.cuh - common includes of the learned SGS correction's CNN kernels.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/lexgb.h"
