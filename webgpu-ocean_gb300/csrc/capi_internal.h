// capi_internal.h -- what the C ABI's translation units share: error
// reporting, the device guard, host record transfers, scene constants, the
// task-size autotuner and the batch handle (capi.cu: simulator and scene
// builders; capi_batch.cu: batches; capi_adjoint.cu: differentiation).
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mpm.h"
#include "mpm_internal.h"
#include "sorted_engine.h"

namespace mpm {

// The message mpm_last_error() returns (capi.cu).
void set_last_error(const std::string& msg);

inline int fail(int code, const std::string& msg) {
    set_last_error(msg);
    return code;
}

inline int cuda_fail(cudaError_t e, const char* what) {
    return fail(MPM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define MPM_CUDA(call)                                   \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// Switches to the handle's device for the duration of a call.
struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) { ok = false; return; }
        if (prev != dev && cudaSetDevice(dev) != cudaSuccess) ok = false;
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

// Host 80-byte records <-> device particle streams through a staging buffer
// (capi.cu).
cudaError_t upload_records(const Particles& dst, const float* host, int n, float* stage,
                           cudaStream_t st);
cudaError_t download_records(const Particles& src, float* host, int n, float* stage,
                             cudaStream_t st);

// WGSL i32(f32): truncation toward zero, saturating, NaN -> 0 (capi.cu).
int f2i_trunc_sat(float x);
// mls-mpm.ts:229 gridCount (capi.cu).
long long grid_count_of(const float b[3]);
// SimConsts of one scene; MPM_OK or an error for an unusable description
// (capi_batch.cu).
int scene_consts(const mpm_scene_desc& d, SimConsts& k);

// Times `substeps` sorted-engine substeps for each combination of z-pair
// threshold, task-kernel block size, task size and lane-table threshold from
// the same saved state and keeps the fastest.  Each candidate first runs once untimed, so that
// the CUDA graphs the timed run replays are captured outside it.  The state
// after the call is the state before it (particles, posvel, counters, grid).
template <class StepFn>
int tune_engine(SortedEngine* e, ParticleStore& ps, int n, float4* posvel,
                unsigned long long* counters, int substeps, cudaStream_t st, StepFn step,
                int* chosen, int* chosen_lane, double* ms_out, int* chosen_threads = nullptr) {
    static const int kPairs[] = {0, 256, 512, 1 << 30};
    static const int kThreads[] = {128, 256, 512};
    static const int kCaps[] = {128, 256, 512, 1024};
    static const int kLanes[] = {32, 128, 512, 1 << 30};  // 1 << 30: no lane table
    Particles save{};
    float4* pv = nullptr;
    unsigned long long cnt[2] = {0, 0};
    cudaEvent_t a = nullptr, b = nullptr;
    auto cleanup = [&]() {
        cudaFree(save.p0); cudaFree(save.p1); cudaFree(save.p2); cudaFree(save.p3);
        cudaFree(pv);
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    };
    cudaError_t err = cudaSuccess;
    float4** sp[4] = {&save.p0, &save.p1, &save.p2, &save.p3};
    for (int q = 0; q < 4 && err == cudaSuccess; ++q) err = cudaMalloc(sp[q], sizeof(float4) * (size_t)(n ? n : 1));
    if (err == cudaSuccess) err = cudaMalloc(&pv, sizeof(float4) * 2 * (size_t)(n ? n : 1));
    if (err == cudaSuccess) err = cudaEventCreate(&a);
    if (err == cudaSuccess) err = cudaEventCreate(&b);
    if (err == cudaSuccess) err = cudaMemcpy(cnt, counters, sizeof(cnt), cudaMemcpyDeviceToHost);
    // canonical snapshot of the state
    if (err == cudaSuccess) {
        const int c = ps.cur;
        if (ps.canonical) {
            const float4* src[4] = {ps.P[c].p0, ps.P[c].p1, ps.P[c].p2, ps.P[c].p3};
            for (int q = 0; q < 4 && err == cudaSuccess; ++q)
                err = cudaMemcpyAsync(*sp[q], src[q], sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, st);
        } else {
            launch_canonicalize(ps.P[c], ps.id[c], save, nullptr, n, st);
            err = cudaGetLastError();
        }
    }
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(pv, posvel, sizeof(float4) * 2 * (size_t)n, cudaMemcpyDeviceToDevice, st);
    auto restore = [&]() -> cudaError_t {
        ps.cur = 0;
        ps.canonical = true;
        const float4* src[4] = {save.p0, save.p1, save.p2, save.p3};
        float4* dst[4] = {ps.P[0].p0, ps.P[0].p1, ps.P[0].p2, ps.P[0].p3};
        for (int q = 0; q < 4; ++q) {
            cudaError_t e2 = cudaMemcpyAsync(dst[q], src[q], sizeof(float4) * (size_t)n, cudaMemcpyDeviceToDevice, st);
            if (e2 != cudaSuccess) return e2;
        }
        launch_iota(ps.id[0], n, st);
        sorted_invalidate(e);
        return cudaGetLastError();
    };
    int best = 0, best_lane = 0, best_threads = 0, best_pair = 0;
    double best_ms = 0.0;
    for (int pair : kPairs)
    for (int th : kThreads)
    for (int cap : kCaps) {
        for (int lane : kLanes) {
            if (err != cudaSuccess) break;
            if (sorted_set_pair_max(e, pair) != 0 || sorted_set_threads(e, th) != 0 ||
                sorted_set_task_cap(e, cap) != 0 || sorted_set_lane_table_min(e, lane) != 0)
                continue;
            if ((err = restore()) != cudaSuccess) break;
            if (step(1) != 0 || step(substeps) != 0) { err = cudaErrorLaunchFailure; break; }
            if ((err = restore()) != cudaSuccess) break;
            if (step(1) != 0) { err = cudaErrorLaunchFailure; break; }  // primes
            cudaEventRecord(a, st);
            if (step(substeps) != 0) { err = cudaErrorLaunchFailure; break; }
            cudaEventRecord(b, st);
            if ((err = cudaEventSynchronize(b)) != cudaSuccess) break;
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (!best || ms < best_ms) {
                best = cap;
                best_lane = lane;
                best_threads = th;
                best_pair = pair;
                best_ms = ms;
            }
        }
    }
    if (err == cudaSuccess) err = restore();
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(posvel, pv, sizeof(float4) * 2 * (size_t)n, cudaMemcpyDeviceToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(counters, cnt, sizeof(cnt), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cleanup();
    if (err != cudaSuccess) return cuda_fail(err, "autotune");
    if (best) {
        sorted_set_pair_max(e, best_pair);
        sorted_set_threads(e, best_threads);
        sorted_set_task_cap(e, best);
        sorted_set_lane_table_min(e, best_lane);
    }
    if (chosen) *chosen = best;
    if (chosen_lane) *chosen_lane = best_lane;
    if (chosen_threads) *chosen_threads = best_threads;
    if (ms_out) *ms_out = best_ms;
    return MPM_OK;
}

}  // namespace mpm

struct mpm_batch {
    int device = 0;
    std::vector<mpm_scene_desc> desc;
    std::vector<mpm::SimConsts> consts;
    std::vector<long long> first;  // first particle of each scene
    int n = 0;
    mpm::ParticleStore ps{};
    float4* posvel = nullptr;
    unsigned long long* counters = nullptr;  // [0] out-of-range, [1] non-finite scratch
    mpm::SortedEngine* sorted = nullptr;
    bool graph = true;
    bool stepped = false;
    mpm::LaunchProfiler prof;
};

namespace mpm {
int check_batch(const mpm_batch* b);  // capi_batch.cu
}  // namespace mpm
