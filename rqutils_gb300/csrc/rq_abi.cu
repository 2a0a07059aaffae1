// Host helpers of the C ABI: error state, device properties, scratch sizing, version.
#include <atomic>
#include <cstdio>
#include <mutex>
#include <string>

#include "rq_common.cuh"
#include "rq_host.h"

namespace rq {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string &msg) { g_last_error = msg; }

int fail(int code, const std::string &msg) {
    set_error(msg);
    return code;
}

int cuda_fail(cudaError_t e, const char *what) {
    return fail(RQ_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int sm_count() {
    // per device; atomic so that threads querying at once do not race on the entry
    static std::atomic<int> cached[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int n = cached[dev].load(std::memory_order_relaxed);
    if (n == 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 152;
        cached[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

size_t scratch_scan_offset() { return kScratchReduce + reduce_scratch_bytes(); }

size_t scratch_bytes(int64_t D) {
    const int64_t nblk = (D + 1023) / 1024 + 1;
    return scratch_scan_offset() + (size_t)nblk * sizeof(int64_t) + 64;
}

int vtype_size(int32_t vtype) {
    switch (vtype) {
        case RQ_F32: return 4;
        case RQ_F64: return 8;
        case RQ_C64: return 8;
        case RQ_C128: return 16;
        default: return 0;
    }
}

}  // namespace rq

RQ_API const char *rq_last_error(void) { return rq::g_last_error.c_str(); }

RQ_API int rq_version(void) { return 100; }

RQ_API int rq_scratch_size(int64_t D, size_t *bytes) {
    if (!bytes || D < 0) return rq::fail(RQ_E_ARG, "rq_scratch_size: bad arguments");
    *bytes = rq::scratch_bytes(D);
    return RQ_OK;
}
