// mpm_internal.h -- library-internal types shared by the .cu files.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "mpm_math.cuh"

namespace mpm {

// Two sets of particle streams plus the particle id held by each slot.  P[cur]
// holds the current state; when `canonical`, slot i holds particle i (the
// sorted engine keeps particles physically in bin order between substeps).
struct ParticleStore {
    Particles P[2];
    uint32_t* id[2];
    int cur = 0;
    bool canonical = true;
};

// Kernel ids for launch accounting (names in kernel_name()).
enum KernelId {
    KID_CLEAR_GRID = 0,
    KID_P2G_1,
    KID_P2G_2,
    KID_UPDATE_GRID,
    KID_G2P,
    KID_COPY_POSITION,
    KID_BIN,
    KID_SCAN,
    KID_SCATTER,
    KID_SORTED_P2G_1,
    KID_SORTED_P2G_2,
    KID_SORTED_G2P_P2G_1,
    KID_EXPORT,
    KID_CANONICALIZE,
    KID_COUNT
};

const char* kernel_name(int id);

// Counts every kernel launch and, when enabled, brackets each with CUDA
// events recorded on the launch stream (per-kernel device time).
struct LaunchProfiler {
    bool enabled = false;
    long long launches[KID_COUNT] = {};
    double total_ms[KID_COUNT] = {};
    long long timed[KID_COUNT] = {};
    struct Pending {
        int id;
        cudaEvent_t a, b;
    };
    Pending* pending = nullptr;
    int npending = 0, cap = 0;
    cudaEvent_t* pool = nullptr;
    int npool = 0, pool_cap = 0;
    cudaEvent_t open = nullptr;

    void before(cudaStream_t st);
    void after(int id, cudaStream_t st);
    int collect();  // waits for pending events and accumulates; 0 on success
    void reset();
    void release();
};

// Every launcher takes the stream it runs on; none synchronises.
// Dispatch engine: one kernel per WGSL entry point (reference order).
void launch_clear_grid(int4* cells, int grid_count, cudaStream_t st);
void launch_p2g_1(const Particles& P, int4* cells, const SimConsts& k,
                  unsigned long long* oob, cudaStream_t st);
void launch_p2g_2(const Particles& P, int4* cells, const SimConsts& k,
                  unsigned long long* oob, cudaStream_t st);
void launch_update_grid(int4* cells, const SimConsts& k, cudaStream_t st);
void launch_g2p(const Particles& P, const int4* cells, const SimConsts& k,
                unsigned long long* oob, cudaStream_t st);
void launch_copy_position(const Particles& P, float4* posvel, int n, cudaStream_t st);

// dst[id[j]] = src[j] for j < n, and id_dst[i] = i.
void launch_canonicalize(const Particles& src, const uint32_t* id, const Particles& dst,
                         uint32_t* id_dst, int n, cudaStream_t st);
void launch_iota(uint32_t* id, int n, cudaStream_t st);
// 80-byte reference records (device, 16-byte aligned) <-> particle streams.
void launch_records_to_streams(const float* rec, const Particles& P, int n, cudaStream_t st);
void launch_streams_to_records(const Particles& P, float* rec, int n, cudaStream_t st);

// Diagnostics.
void launch_count_nonfinite(const Particles& P, int n, unsigned long long* out, cudaStream_t st);
void launch_packed_probe(const float* a, const float* b, int npairs, float* out6);
void launch_convert_probe(const float* in, int n, float fm, int* enc_out, float* dec_out,
                          cudaStream_t st);

}  // namespace mpm
