// noalloc.cu -- mpm_count_nonfinite_noalloc: the watchdog scan behind
// mpm_check_health, for callers that cannot allocate device memory.
//
// Who cannot allocate: a host that calls into this library from a frame
// loop (WebGPU-Ocean drives execute() once per animation frame) or from a
// plugin host that owns all device memory through its own allocator.
// cudaMalloc and cudaFree may synchronize the whole device and take
// unbounded time, which a fixed per-frame budget cannot absorb, and such
// hosts hand the library pre-allocated buffers only.  This entry point
// therefore takes the caller's buffers and keeps its scratch (one partial
// count per thread block and a completion ticket) in a file-scope device
// array that is part of the library image: every GPU that loads libmpm.so
// holds those 512 KiB until the process exits.
//
// Which floats are checked: for the 80-byte particle record (stride 20) the
// 16 state floats, as mpm_check_health does; the five padding floats (3, 7,
// 11, 15, 19: the fourth float of each vec3f slot and of each column of C)
// are skipped, because a WGSL struct store leaves them unspecified.  For any
// other stride every float of a record is checked.
#include <cuda_runtime.h>

#include <string>

#include "../../include/mpm.h"

namespace mpm {
void set_last_error(const std::string& msg);  // capi.cu: read back by mpm_last_error()
}

namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 65536;  // records per call <= kMaxBlocks * kThreads
constexpr long long kMaxRecords = (long long)kMaxBlocks * kThreads;

// [0]: completion ticket, zero between calls; [1 + b]: count of block b.
static __device__ __align__(256) unsigned long long g_scratch[1 + kMaxBlocks];

// g_scratch is zero when the module loads into a context, and the last block
// of every call sets the ticket back to zero, so no call has to clear it.

__global__ void __launch_bounds__(kThreads)
    k_count_nonfinite_noalloc(const float* __restrict__ rec, int stride, int n,
                              unsigned long long* __restrict__ scratch,
                              int64_t* __restrict__ count_out) {
    __shared__ unsigned s_count;
    __shared__ unsigned long long s_warp[kThreads / 32];
    __shared__ bool s_last;
    if (threadIdx.x == 0) s_count = 0u;
    __syncthreads();
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    bool bad = false;
    if (i < n) {
        const float* r = rec + i * (long long)stride;
        const bool padded = stride == 20;  // the reference's 80-byte particle record
        for (int j = 0; j < stride; ++j)
            if (!padded || (j & 3) != 3) bad |= !isfinite(r[j]);
    }
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31u) == 0 && m) atomicAdd(&s_count, (unsigned)__popc(m));
    __syncthreads();
    if (threadIdx.x == 0) {
        scratch[1 + blockIdx.x] = s_count;
        __threadfence();
        s_last = atomicAdd(&scratch[0], 1ull) == (unsigned long long)(gridDim.x - 1);
    }
    __syncthreads();
    if (!s_last) return;
    // The last block to finish adds up every block's count.
    __threadfence();
    unsigned long long sum = 0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads) sum += __ldcg(&scratch[1 + b]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xffffffffu, sum, o);
    if ((threadIdx.x & 31u) == 0) s_warp[threadIdx.x >> 5] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long total = 0;
        for (int w = 0; w < kThreads / 32; ++w) total += s_warp[w];
        *count_out = (int64_t)total;
        scratch[0] = 0ull;  // the next call's ticket starts at zero
    }
}

int fail(int code, const std::string& msg) {
    mpm::set_last_error(msg);
    return code;
}

// The device address of g_scratch in the current device's context.  In host
// code the array's name is only a host-side stand-in, not a device address.
// The lookup runs on every call (it allocates nothing), so a context that
// was reset or replaced on the same device never leaves a stale address.
int scratch_for_current_device(unsigned long long** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(MPM_E_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess)
        return fail(MPM_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
    *out = static_cast<unsigned long long*>(p);
    return MPM_OK;
}

}  // namespace

extern "C" int mpm_count_nonfinite_noalloc(const float* records, int stride_floats, int n,
                                           int64_t* count_out, void* stream) {
    if (n < 0 || stride_floats < 1 || !count_out || (n > 0 && !records))
        return fail(MPM_E_INVALID, "mpm_count_nonfinite_noalloc: bad arguments");
    if ((long long)n > kMaxRecords)
        return fail(MPM_E_CAPACITY,
                    "mpm_count_nonfinite_noalloc: at most 16,777,216 records per call "
                    "(its scratch is a fixed 512 KiB device array)");
    unsigned long long* scratch = nullptr;
    if (int rc = scratch_for_current_device(&scratch)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n == 0) {
        const cudaError_t e = cudaMemsetAsync(count_out, 0, sizeof(int64_t), st);
        if (e != cudaSuccess) return fail(MPM_E_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
        return MPM_OK;
    }
    const int blocks = (int)((n + kThreads - 1) / kThreads);
    k_count_nonfinite_noalloc<<<blocks, kThreads, 0, st>>>(records, stride_floats, n, scratch,
                                                           count_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MPM_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return MPM_OK;
}
