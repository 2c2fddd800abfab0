// Host-side glue between the renderer context (sglc_api.cu) and the neural shader objects
// (sglc_nn.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "softgl_cuda.h"

namespace sglc {

cudaStream_t ctxStream(sglc_context *ctx);
int ctxDevice(sglc_context *ctx);
void ctxSetError(sglc_context *ctx, const char *msg);
// records == null stops capturing
void ctxSetCapture(sglc_context *ctx, float *records, unsigned long long *count, long long capacity, int stride);
// forget every reference to a network that is being destroyed (program bindings, capture)
void ctxDetachNeural(sglc_context *ctx, const sglc_neural *net);
const uint8_t *neuralImage(const sglc_neural *net);

}  // namespace sglc
