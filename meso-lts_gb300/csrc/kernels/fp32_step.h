// Host-visible interface of the FP32-storage Shakhov step (fp32_step.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "device_common.cuh"

namespace meso {

struct Fp32State {
    int enabled = 0;
};

}  // namespace meso
