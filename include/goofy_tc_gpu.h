// goofy_tc_gpu.h -- drop-in replacement declarations for the reference's
// public API (GoofyTC/goofy_tc.h:10-13).  Same namespace, names, signatures,
// argument meaning and return codes:
//   0 on success, -1 when width % 16 != 0, -2 when height % 4 != 0
//   (goofy_tc.h:1500-1508).
// The bodies live in libgoofy_gb300.so and run on the GPU (no CPU fallback);
// on a CUDA failure they return the negative GOOFY_ERR_* code of goofy_gpu.h
// instead of encoding on the CPU.
#pragma once

#include "goofy_gpu.h"

namespace goofy {
int compressDXT1(unsigned char* result, const unsigned char* input, unsigned int width, unsigned int height,
                 unsigned int stride);
int compressETC1(unsigned char* result, const unsigned char* input, unsigned int width, unsigned int height,
                 unsigned int stride);
}  // namespace goofy
