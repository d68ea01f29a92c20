// Device scratch buffers of a context, and the allocation-failure injection
// used by the failure-detection tests.
//
// A DevBuf grows on demand and is kept between calls. Growing waits for all
// queued work first, since kernels of earlier calls may still read the old
// allocation. A failed allocation leaves the buffer empty and returns
// RFBA_ERR_NOMEM (cudaMalloc out of memory) or RFBA_ERR_CUDA, with the buffer's
// name in the error text; the next call simply tries again.
//
// RFBA_TEST_ALLOC_FAIL=k (k >= 1) makes the k-th buffer allocation counted from
// the moment the variable takes that value fail as an out-of-memory would,
// once; allocations before and after it are unaffected. The variable is read
// at every allocation, so a test can set it, make one call and clear it.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <string>

#include "../../include/rfba_srrf.h"

namespace rfba {

void set_error(const std::string& msg);

// True when this allocation is the one RFBA_TEST_ALLOC_FAIL names.
inline bool injected_alloc_failure() {
    static std::mutex mu;
    static std::string seen;
    static long long count = 0;
    static bool fired = false;
    const char* e = std::getenv("RFBA_TEST_ALLOC_FAIL");
    const std::string v = e ? e : "";
    std::lock_guard<std::mutex> lk(mu);
    if (v != seen) {
        seen = v;
        count = 0;
        fired = false;
    }
    if (v.empty() || fired) return false;
    const long long k = std::atoll(v.c_str());
    if (k < 1) return false;
    if (++count == k) {
        fired = true;
        return true;
    }
    return false;
}

struct DevBuf {
    void* p = nullptr;
    size_t n = 0;
    int ensure(size_t bytes, const char* what) {
        if (bytes <= n) return RFBA_OK;
        if (p) {
            cudaDeviceSynchronize();
            cudaFree(p);
        }
        p = nullptr;
        n = 0;
        const size_t want = std::max(bytes, (size_t)256);
        if (injected_alloc_failure()) {
            set_error(std::string(what) + ": out of memory (injected by RFBA_TEST_ALLOC_FAIL)");
            return RFBA_ERR_NOMEM;
        }
        const cudaError_t e = cudaMalloc(&p, want);
        if (e != cudaSuccess) {
            p = nullptr;
            cudaGetLastError();
            set_error(std::string(what) + ": " + cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? RFBA_ERR_NOMEM : RFBA_ERR_CUDA;
        }
        n = want;
        return RFBA_OK;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
};

}  // namespace rfba
