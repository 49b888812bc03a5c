// wlc_attr.h -- kernel attributes, which CUDA keeps per device.
//
// cudaFuncSetAttribute(MaxDynamicSharedMemorySize) applies to the device
// that is current when it is called.  A process that launches on several
// devices (one context per device, or the allocation-free step on each
// GPU) must set it once per (kernel, device); a single process-wide flag
// would leave every device but the first at the 48 KB default and make
// their large-shared-memory launches fail.
#pragma once
#include <cuda_runtime.h>

#include <mutex>
#include <set>
#include <utility>

namespace wlc {

// Raise the dynamic shared-memory limit of kernel `fn` to `bytes` on the
// current device, once per (kernel, device).  Thread-safe; returns the
// error of cudaGetDevice / cudaFuncSetAttribute (nothing is recorded on
// failure, so a later call retries).
inline cudaError_t smem_attr_once(const void* fn, int bytes) {
    static std::mutex mu;
    static std::set<std::pair<const void*, int>> done;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({fn, dev})) return cudaSuccess;
    e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e == cudaSuccess) done.insert({fn, dev});
    return e;
}

template <typename K> inline cudaError_t smem_attr_once(K* fn, int bytes) {
    return smem_attr_once(reinterpret_cast<const void*>(fn), bytes);
}

}  // namespace wlc
