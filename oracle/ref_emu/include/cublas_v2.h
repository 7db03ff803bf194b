// cuBLAS v2 header of the CPU emulation (TEST INFRASTRUCTURE ONLY).
#pragma once
#include "cublas_api.h"
