// Host-side helpers shared by the entry points: error reporting, CUDA checks, launch sizing,
// scratch layout.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "rqsqd.h"

#define RQ_API extern "C" __attribute__((visibility("default")))

namespace rq {

// Thread-local last error message (rq_last_error).
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

// Returns RQ_E_CUDA with a message if `e` is an error.
int cuda_fail(cudaError_t e, const char *what);

#define RQ_CUDA(call)                                                 \
    do {                                                              \
        cudaError_t e_ = (call);                                      \
        if (e_ != cudaSuccess) return ::rq::cuda_fail(e_, #call);     \
    } while (0)

#define RQ_TRY(call)                                                  \
    do {                                                              \
        int rc_ = (call);                                             \
        if (rc_ != RQ_OK) return rc_;                                 \
    } while (0)

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// Number of SMs of the current device (cached per device).
int sm_count();

// Scratch layout (bytes from the scratch base):
//   [0, 16)         reserved
//   [16, 32)        device error flag (int32)
//   [32, 32 + R)    grid-reduction area (its counter, then the partials), R = reduce_scratch_bytes()
//   [.., ..)        scan block sums for D rows (int64)
constexpr size_t kScratchErr = 16;
constexpr size_t kScratchReduce = 32;
size_t scratch_scan_offset();
size_t scratch_bytes(int64_t D);

inline int *scratch_err(void *scratch) {
    return reinterpret_cast<int *>(static_cast<char *>(scratch) + kScratchErr);
}
inline void *scratch_reduce(void *scratch) {
    return static_cast<char *>(scratch) + kScratchReduce;
}
inline int64_t *scratch_scan(void *scratch) {
    return reinterpret_cast<int64_t *>(static_cast<char *>(scratch) + scratch_scan_offset());
}

int vtype_size(int32_t vtype);

// Launch settings of one kernel: the dynamic shared memory it has been opted into and its
// occupancy at one shared-memory size.  Each launcher keeps one entry per host thread and device
// (cache_slot), so threads never share an entry and devices with different SM counts or
// attributes never see each other's values.
struct KernelLaunchCache {
    size_t configured = 0;
    size_t occ_smem = ~size_t(0);
    int occ_blocks = 1;
};
constexpr int kMaxCachedDevices = 64;

// Opt kern into smem bytes of dynamic shared memory (a kernel with static shared memory can need
// the opt-in below 48 KB of dynamic memory too) and return its resident blocks per SM at `block`
// threads, querying the runtime only when `c` does not hold the answer yet (the occupancy query
// is also reached while a stream is being captured, where only stream work should be issued).
template <typename KernT>
int configure_kernel(KernT kern, KernelLaunchCache &c, size_t smem, int block, int *per_sm) {
    if (smem > c.configured) {
        RQ_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        c.configured = smem;
    }
    if (c.occ_smem != smem) {
        int per = 0;
        RQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, block, smem));
        c.occ_blocks = per < 1 ? 1 : per;
        c.occ_smem = smem;
    }
    *per_sm = c.occ_blocks;
    return RQ_OK;
}

// This thread's entry for the current device in a launcher's table.
inline int cache_slot(KernelLaunchCache (&table)[kMaxCachedDevices], KernelLaunchCache **out) {
    int dev = 0;
    RQ_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxCachedDevices) return fail(RQ_E_RANGE, "device index out of range");
    *out = &table[dev];
    return RQ_OK;
}

}  // namespace rq
