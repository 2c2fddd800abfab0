// Host-side helpers shared by the C-ABI translation units: a scoped device switch and a
// per-device, thread-safe "set this kernel attribute once" record.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

namespace sglc {

// Makes `device` current for the enclosing scope and restores the caller's device on exit. Every
// entry point that touches a context's memory or stream holds one, so a context may be driven from
// any host thread whatever that thread's current device is.
class DeviceGuard {
 public:
  explicit DeviceGuard(int device) {
    if (device < 0) return;
    if (cudaGetDevice(&prev_) != cudaSuccess) {
      cudaGetLastError();
      prev_ = -1;
    }
    if (prev_ != device && cudaSetDevice(device) == cudaSuccess) switched_ = true;
  }
  ~DeviceGuard() {
    if (switched_ && prev_ >= 0) cudaSetDevice(prev_);
  }
  DeviceGuard(const DeviceGuard &) = delete;
  DeviceGuard &operator=(const DeviceGuard &) = delete;

 private:
  int prev_ = -1;
  bool switched_ = false;
};

// A function attribute (here: the dynamic shared-memory limit) belongs to a kernel on one device.
// The first launch on each device sets it, under std::call_once so that contexts on several host
// threads may race to it; the result is kept per device and returned to every later caller.
constexpr int kMaxDevices = 64;

struct PerDeviceAttr {
  std::once_flag once[kMaxDevices];
  cudaError_t err[kMaxDevices] = {};
};

template <class Kernel>
inline cudaError_t setDynamicSmemOnce(PerDeviceAttr &a, Kernel *kernel, int bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  std::call_once(a.once[dev], [&] {
    a.err[dev] = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  });
  return a.err[dev];
}

// streaming multiprocessors of the current device (152 on a GB300), for grids sized in whole waves
inline int currentSmCount() {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      sms <= 0) {
    cudaGetLastError();
    return 152;
  }
  return sms;
}

}  // namespace sglc
