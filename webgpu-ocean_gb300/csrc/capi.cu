// capi.cu -- the C ABI of libmpm.so (include/mpm.h): simulator handle,
// device memory, scene builders and the per-frame stage sequencing of
// MLSMPMSimulator (mls-mpm/mls-mpm.ts:12-276).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/mpm.h"
#include "adjoint.h"
#include "mpm_internal.h"
#include "sorted_engine.h"

using namespace mpm;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
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

// ---------------------------------------------------------------------------
// Scene builders (host).  Doubles throughout, as JS numbers; this file is
// compiled with -ffp-contract=off so each double operation rounds alone.
// ---------------------------------------------------------------------------

struct SplitMix64 {
    uint64_t s;
    explicit SplitMix64(uint64_t seed) : s(seed) {}
    uint64_t next() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double random() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// initDambreak, mls-mpm/mls-mpm.ts:195-223.
int scene_dambreak(float* out, int max_particles, const double box[3], uint64_t seed) {
    SplitMix64 rng(seed);
    const double spacing = 0.65;
    int n = 0;
    for (double j = 0; j < box[1] * 0.80 && n < max_particles; j += spacing) {
        for (double i = 3; i < box[0] - 4 && n < max_particles; i += spacing) {
            for (double k = 3; k < box[2] / 2 && n < max_particles; k += spacing) {
                const double jitter = 2.0 * rng.random();
                float* P = out + 20 * (size_t)n;
                std::memset(P, 0, 80);
                P[0] = (float)(i + jitter);
                P[1] = (float)(j + jitter);
                P[2] = (float)(k + jitter);
                ++n;
            }
        }
    }
    return n;
}

int scene_lattice(float* out, int npa, double origin, double spacing, double jitter,
                  uint64_t seed) {
    SplitMix64 rng(seed);
    size_t p = 0;
    for (int ix = 0; ix < npa; ++ix)
        for (int iy = 0; iy < npa; ++iy)
            for (int iz = 0; iz < npa; ++iz) {
                float* P = out + 20 * p;
                std::memset(P, 0, 80);
                const int idx[3] = {ix, iy, iz};
                for (int a = 0; a < 3; ++a) {
                    const double u = rng.random();
                    const double x = (origin + spacing * (double)idx[a]) + jitter * (2.0 * u - 1.0);
                    P[a] = (float)x;
                }
                ++p;
            }
    return (int)p;
}

// Reference 80-byte records in host memory <-> the library's four float4
// streams, converted on the device: one copy of the records through a
// staging buffer of 80 bytes per particle (`stage`, or a stream-ordered
// allocation when null), then a gather kernel.
struct Stage {
    float* p = nullptr;
    bool owned = false;
    cudaError_t get(float* given, int n, cudaStream_t st) {
        if (given) {
            p = given;
            return cudaSuccess;
        }
        owned = true;
        return cudaMallocAsync(reinterpret_cast<void**>(&p), (size_t)80 * (size_t)n, st);
    }
    void release(cudaStream_t st) {
        if (owned && p) cudaFreeAsync(p, st);
        p = nullptr;
        owned = false;
    }
};

cudaError_t upload_records(const Particles& dst, const float* host, int n, float* stage,
                           cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    Stage sg;
    cudaError_t e = sg.get(stage, n, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sg.p, host, (size_t)80 * (size_t)n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        launch_records_to_streams(sg.p, dst, n, st);
        e = cudaGetLastError();
    }
    sg.release(st);
    return e;
}

cudaError_t download_records(const Particles& src, float* host, int n, float* stage,
                             cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    Stage sg;
    cudaError_t e = sg.get(stage, n, st);
    if (e == cudaSuccess) {
        launch_streams_to_records(src, sg.p, n, st);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host, sg.p, (size_t)80 * (size_t)n, cudaMemcpyDeviceToHost, st);
    sg.release(st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

int f2i_trunc_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int)x;
}

}  // namespace

namespace mpm {
// Lets other translation units report a message through mpm_last_error().
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace mpm

// ---------------------------------------------------------------------------
// The handle
// ---------------------------------------------------------------------------

struct mpm_sim {
    int device = 0;
    mpm_params params{};
    int max_particles = 0;
    long long max_cells = 0;
    float render_diameter = 0.f;

    int n = 0;
    long long grid_count = 0;
    float init_box[3] = {0, 0, 0};
    float real_box[3] = {0, 0, 0};
    bool loaded = false;

    ParticleStore ps{};
    // The reference's cell buffer (x-major, mls-mpm.ts:126-130): the dispatch
    // engine works in it; the sorted engine exports into it on demand.
    int4* grid_ref = nullptr;
    bool ref_current = true;   // false: the sorted engine holds the newest grid
    bool sorted_ok = false;    // the sorted engine can run this scene
    float4* posvel = nullptr;
    bool posvel_owned = false;
    unsigned long long* counters = nullptr;  // [0] out-of-range, [1] non-finite scratch

    float gravity[3] = {0.0f, -0.3f, 0.0f};  // updateGrid.wgsl:34
    bool graph = true;
    int engine = MPM_ENGINE_DISPATCH;
    SortedEngine* sorted = nullptr;
    cudaStream_t internal = nullptr;
    LaunchProfiler prof;
    // pipelined posvel read-back (mpm_download_posvel_async), made on first use
    float4* posvel_snap = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t snap_taken = nullptr, snap_copied = nullptr;

    SimConsts consts() const {
        SimConsts k{};
        k.stiffness = params.stiffness;
        k.rest_density = params.rest_density;
        k.dynamic_viscosity = params.dynamic_viscosity;
        k.dt = params.dt;
        k.fm = params.fixed_point_multiplier;
        for (int a = 0; a < 3; ++a) {
            k.init_box[a] = init_box[a];
            k.real_box[a] = real_box[a];
        }
        k.Y = f2i_trunc_sat(init_box[1]);
        k.Z = f2i_trunc_sat(init_box[2]);
        k.grid_count = (int)grid_count;
        k.n = n;
        for (int a = 0; a < 3; ++a) k.gravity[a] = gravity[a];
        return k;
    }
};

namespace {

int check_sim(const mpm_sim* s) {
    if (!s) return fail(MPM_E_INVALID, "null simulator handle");
    return MPM_OK;
}

// mls-mpm.ts:229 gridCount = ceil(X) * ceil(Y) * ceil(Z)
long long grid_count_of(const float b[3]) {
    return (long long)std::ceil((double)b[0]) * (long long)std::ceil((double)b[1]) *
           (long long)std::ceil((double)b[2]);
}

int load_particles(mpm_sim* s, const float* aos80, int n, const float init_box[3]) {
    if (n < 0) return fail(MPM_E_INVALID, "negative particle count");
    if (n > s->max_particles)
        return fail(MPM_E_CAPACITY, "numParticles exceeds the particle capacity");
    for (int a = 0; a < 3; ++a)
        if (!(init_box[a] >= 0.f) || !std::isfinite(init_box[a]))
            return fail(MPM_E_INVALID, "init box size must be finite and non-negative");
    const long long gc = grid_count_of(init_box);
    if (gc > s->max_cells)
        return fail(MPM_E_GRID_CAPACITY, "gridCount should be equal to or less than maxGridCount");
    if (gc > 0x7fffffffLL) return fail(MPM_E_GRID_CAPACITY, "gridCount exceeds the i32 index range");
    DeviceGuard g(s->device);
    if (!g.ok) return fail(MPM_E_CUDA, "cannot select the simulator's device");
    MPM_CUDA(cudaDeviceSynchronize());
    s->ps.cur = 0;
    s->ps.canonical = true;
    MPM_CUDA(upload_records(s->ps.P[0], aos80, n, nullptr, nullptr));
    launch_iota(s->ps.id[0], n, nullptr);
    MPM_CUDA(cudaGetLastError());
    s->n = n;
    s->grid_count = gc;
    for (int a = 0; a < 3; ++a) s->init_box[a] = s->real_box[a] = init_box[a];
    MPM_CUDA(cudaMemset(s->grid_ref, 0, sizeof(int4) * (size_t)s->max_cells));
    MPM_CUDA(cudaMemset(s->counters, 0, sizeof(unsigned long long) * 2));
    if (n) MPM_CUDA(cudaMemset(s->posvel, 0, sizeof(float4) * 2 * (size_t)n));
    s->ref_current = true;
    s->loaded = true;
    sorted_invalidate(s->sorted);
    s->sorted_ok = sorted_configure(s->sorted, s->consts()) == 0;
    MPM_CUDA(cudaDeviceSynchronize());
    return MPM_OK;
}

// Puts particle i back in slot i (the dispatch engine and the reference
// address particles by index).  Forgets the sorted engine's carried state.
int ensure_canonical(mpm_sim* s, cudaStream_t st) {
    if (s->ps.canonical) return MPM_OK;
    const int c = s->ps.cur;
    s->prof.before(st);
    launch_canonicalize(s->ps.P[c], s->ps.id[c], s->ps.P[c ^ 1], s->ps.id[c ^ 1], s->n, st);
    s->prof.after(KID_CANONICALIZE, st);
    MPM_CUDA(cudaGetLastError());
    s->ps.cur = c ^ 1;
    s->ps.canonical = true;
    sorted_invalidate(s->sorted);
    return MPM_OK;
}

// Brings the reference-layout grid up to date (exports the sorted engine's
// last grid, as updateGrid left it).
int sync_ref_grid(mpm_sim* s, cudaStream_t st) {
    if (s->ref_current) return MPM_OK;
    if (sorted_has_grid(s->sorted)) {
        if (sorted_export_grid(s->sorted, s->consts(), s->grid_ref, st, &s->prof) != 0)
            return fail(MPM_E_CUDA, std::string("sorted engine: ") + sorted_error());
    }
    s->ref_current = true;
    return MPM_OK;
}

// One reference substep on the dispatch engine (mls-mpm.ts:248-265).
void dispatch_kernel(mpm_sim* s, int kernel, const SimConsts& k, cudaStream_t st) {
    int4* cells = s->grid_ref;
    const Particles& P = s->ps.P[s->ps.cur];
    s->prof.before(st);
    switch (kernel) {
        case MPM_KERNEL_CLEAR_GRID: launch_clear_grid(cells, k.grid_count, st); break;
        case MPM_KERNEL_P2G_1: launch_p2g_1(P, cells, k, s->counters, st); break;
        case MPM_KERNEL_P2G_2: launch_p2g_2(P, cells, k, s->counters, st); break;
        case MPM_KERNEL_UPDATE_GRID: launch_update_grid(cells, k, st); break;
        case MPM_KERNEL_G2P: launch_g2p(P, cells, k, s->counters, st); break;
        case MPM_KERNEL_COPY_POSITION: launch_copy_position(P, s->posvel, k.n, st); break;
    }
    s->prof.after(kernel, st);  // MPM_KERNEL_* == KID_* for the six entry points
}

void dispatch_substep(mpm_sim* s, const SimConsts& k, cudaStream_t st) {
    for (int kernel = MPM_KERNEL_CLEAR_GRID; kernel <= MPM_KERNEL_COPY_POSITION; ++kernel)
        dispatch_kernel(s, kernel, k, st);
}

}  // namespace

extern "C" {

void mpm_default_params(mpm_params* out) {
    if (!out) return;
    out->stiffness = 3.0f;
    out->rest_density = 4.0f;
    out->dynamic_viscosity = 0.1f;
    out->dt = 0.2f;
    out->fixed_point_multiplier = 1e7f;
}

int mpm_create(const mpm_params* params, int max_particles, int max_grid_x, int max_grid_y,
               int max_grid_z, float render_diameter, void* posvel_device, size_t posvel_bytes,
               mpm_sim** out) {
    if (!out) return fail(MPM_E_INVALID, "out is null");
    *out = nullptr;
    if (max_particles < 0 || max_grid_x <= 0 || max_grid_y <= 0 || max_grid_z <= 0)
        return fail(MPM_E_INVALID, "capacities must be positive");
    const long long max_cells = (long long)max_grid_x * max_grid_y * max_grid_z;
    if (max_cells > 0x7fffffffLL) return fail(MPM_E_INVALID, "grid capacity exceeds i32 indices");
    if (posvel_device && posvel_bytes < (size_t)32 * (size_t)max_particles)
        return fail(MPM_E_INVALID, "posvel buffer smaller than 32 * max_particles bytes");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MPM_E_NO_DEVICE, "no CUDA device");
    }
    mpm_sim* s = new (std::nothrow) mpm_sim();
    if (!s) return fail(MPM_E_INVALID, "out of host memory");
    MPM_CUDA(cudaGetDevice(&s->device));
    if (params) s->params = *params;
    else mpm_default_params(&s->params);
    s->max_particles = max_particles;
    s->max_cells = max_cells;
    s->render_diameter = render_diameter;
    const size_t np = (size_t)(max_particles > 0 ? max_particles : 1);
    cudaError_t e = cudaSuccess;
    for (int b = 0; b < 2; ++b) {
        Particles& P = s->ps.P[b];
        float4** ps[4] = {&P.p0, &P.p1, &P.p2, &P.p3};
        for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaMalloc(ps[k], sizeof(float4) * np);
        if (e == cudaSuccess) e = cudaMalloc(&s->ps.id[b], sizeof(uint32_t) * np);
    }
    if (e == cudaSuccess) e = cudaMalloc(&s->grid_ref, sizeof(int4) * (size_t)max_cells);
    if (e == cudaSuccess) e = cudaMalloc(&s->counters, sizeof(unsigned long long) * 2);
    if (e == cudaSuccess) {
        if (posvel_device) {
            s->posvel = static_cast<float4*>(posvel_device);
        } else {
            e = cudaMalloc(&s->posvel, sizeof(float4) * 2 * np);
            s->posvel_owned = true;
        }
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->internal, cudaStreamNonBlocking);
    if (e == cudaSuccess) {
        e = cudaMemset(s->grid_ref, 0, sizeof(int4) * (size_t)max_cells);
        if (e == cudaSuccess) e = cudaMemset(s->counters, 0, sizeof(unsigned long long) * 2);
    }
    if (e == cudaSuccess) {
        int rc = sorted_create(&s->sorted, max_particles);
        if (rc != 0) e = cudaErrorMemoryAllocation;
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "mpm_create");
        mpm_destroy(s);
        return rc;
    }
    s->engine = MPM_ENGINE_SORTED;
    *out = s;
    return MPM_OK;
}

int mpm_destroy(mpm_sim* s) {
    if (!s) return MPM_OK;
    DeviceGuard g(s->device);
    cudaDeviceSynchronize();
    for (int b = 0; b < 2; ++b) {
        cudaFree(s->ps.P[b].p0);
        cudaFree(s->ps.P[b].p1);
        cudaFree(s->ps.P[b].p2);
        cudaFree(s->ps.P[b].p3);
        cudaFree(s->ps.id[b]);
    }
    cudaFree(s->grid_ref);
    cudaFree(s->counters);
    if (s->posvel_owned) cudaFree(s->posvel);
    if (s->sorted) sorted_destroy(s->sorted);
    if (s->internal) cudaStreamDestroy(s->internal);
    cudaFree(s->posvel_snap);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->snap_taken) cudaEventDestroy(s->snap_taken);
    if (s->snap_copied) cudaEventDestroy(s->snap_copied);
    s->prof.release();
    delete s;
    return MPM_OK;
}

int mpm_reset_dambreak(mpm_sim* s, int num_particles, const double init_box[3], uint64_t seed) {
    if (int rc = check_sim(s)) return rc;
    if (!init_box) return fail(MPM_E_INVALID, "init_box is null");
    if (num_particles < 0) return fail(MPM_E_INVALID, "negative particle count");
    if (num_particles > s->max_particles)
        return fail(MPM_E_CAPACITY, "numParticles exceeds the particle capacity");
    std::vector<float> buf((size_t)20 * (size_t)(num_particles > 0 ? num_particles : 1));
    const int n = scene_dambreak(buf.data(), num_particles, init_box, seed);
    const float box[3] = {(float)init_box[0], (float)init_box[1], (float)init_box[2]};
    return load_particles(s, buf.data(), n, box);
}

int mpm_upload(mpm_sim* s, const float* aos80, int n, const float init_box[3]) {
    if (int rc = check_sim(s)) return rc;
    if (!init_box || (n > 0 && !aos80)) return fail(MPM_E_INVALID, "null pointer");
    return load_particles(s, aos80, n, init_box);
}

int mpm_step(mpm_sim* s, int substeps, void* stream) {
    if (int rc = check_sim(s)) return rc;
    if (!s->loaded) return fail(MPM_E_STATE, "no scene loaded (call reset first)");
    if (substeps < 0) return fail(MPM_E_INVALID, "negative substep count");
    DeviceGuard g(s->device);
    if (!g.ok) return fail(MPM_E_CUDA, "cannot select the simulator's device");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const SimConsts k = s->consts();
    if (s->engine == MPM_ENGINE_DISPATCH || !s->sorted_ok) {
        if (int rc = sync_ref_grid(s, st)) return rc;
        if (int rc = ensure_canonical(s, st)) return rc;
        for (int i = 0; i < substeps; ++i) dispatch_substep(s, k, st);
        if (substeps > 0) sorted_invalidate(s->sorted);
    } else if (substeps > 0) {
        if (sorted_step(s->sorted, &s->ps, s->posvel, s->counters, k, substeps, st, &s->prof,
                        s->graph) != 0)
            return fail(MPM_E_CUDA, std::string("sorted engine: ") + sorted_error());
        s->ref_current = false;
    }
    MPM_CUDA(cudaGetLastError());
    return MPM_OK;
}

int mpm_set_real_box(mpm_sim* s, const float real_box[3]) {
    if (int rc = check_sim(s)) return rc;
    if (!real_box) return fail(MPM_E_INVALID, "real_box is null");
    for (int a = 0; a < 3; ++a) s->real_box[a] = real_box[a];
    return MPM_OK;
}

int mpm_set_gravity(mpm_sim* s, const float gravity[3]) {
    if (int rc = check_sim(s)) return rc;
    if (!gravity) return fail(MPM_E_INVALID, "gravity is null");
    for (int a = 0; a < 3; ++a) s->gravity[a] = gravity[a];
    return MPM_OK;
}

int mpm_set_graph(mpm_sim* s, int enable) {
    if (int rc = check_sim(s)) return rc;
    s->graph = enable != 0;
    return MPM_OK;
}

int mpm_set_task_size(mpm_sim* s, int cap) {
    if (int rc = check_sim(s)) return rc;
    if (sorted_set_task_cap(s->sorted, cap) != 0) return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_get_task_size(const mpm_sim* s) { return s ? sorted_task_cap(s->sorted) : MPM_E_INVALID; }

}  // extern "C"

namespace {
// Times `substeps` sorted-engine substeps for each candidate task size from
// the same saved state and keeps the fastest.  The state after the call is
// the state before it (particles, posvel, counters, grid).
template <class StepFn>
int tune_task_cap(SortedEngine* e, ParticleStore& ps, int n, float4* posvel,
                  unsigned long long* counters, int substeps, cudaStream_t st, StepFn step,
                  int* chosen, double* ms_out) {
    static const int kCands[] = {64, 128, 256, 512, 1024};
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
    int best = 0;
    double best_ms = 0.0;
    for (int cap : kCands) {
        if (err != cudaSuccess) break;
        if (sorted_set_task_cap(e, cap) != 0) continue;
        if ((err = restore()) != cudaSuccess) break;
        if (step(1) != 0) { err = cudaErrorLaunchFailure; break; }  // primes
        cudaEventRecord(a, st);
        if (step(substeps) != 0) { err = cudaErrorLaunchFailure; break; }
        cudaEventRecord(b, st);
        if ((err = cudaEventSynchronize(b)) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (!best || ms < best_ms) { best = cap; best_ms = ms; }
    }
    if (err == cudaSuccess) err = restore();
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(posvel, pv, sizeof(float4) * 2 * (size_t)n, cudaMemcpyDeviceToDevice, st);
    if (err == cudaSuccess) err = cudaMemcpyAsync(counters, cnt, sizeof(cnt), cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaStreamSynchronize(st);
    cleanup();
    if (err != cudaSuccess) return cuda_fail(err, "autotune");
    if (best) sorted_set_task_cap(e, best);
    if (chosen) *chosen = best;
    if (ms_out) *ms_out = best_ms;
    return MPM_OK;
}
}  // namespace

extern "C" {

int mpm_autotune(mpm_sim* s, int substeps, int* chosen_task_size) {
    if (int rc = check_sim(s)) return rc;
    if (!s->loaded) return fail(MPM_E_STATE, "no scene loaded (call reset first)");
    if (substeps < 1) return fail(MPM_E_INVALID, "substeps must be positive");
    if (!s->sorted_ok || s->n == 0) {
        if (chosen_task_size) *chosen_task_size = mpm_get_task_size(s);
        return MPM_OK;
    }
    DeviceGuard g(s->device);
    if (int rc = sync_ref_grid(s, nullptr)) return rc;
    MPM_CUDA(cudaDeviceSynchronize());
    const SimConsts k = s->consts();
    auto step = [&](int ns) {
        return sorted_step(s->sorted, &s->ps, s->posvel, s->counters, k, ns, s->internal, &s->prof,
                           s->graph);
    };
    const int rc = tune_task_cap(s->sorted, s->ps, s->n, s->posvel, s->counters, substeps,
                                 s->internal, step, chosen_task_size, nullptr);
    s->ref_current = true;  // the grid from before the call
    return rc;
}

int mpm_num_particles(const mpm_sim* s) { return s ? s->n : 0; }
int64_t mpm_grid_count(const mpm_sim* s) { return s ? s->grid_count : 0; }
float mpm_render_diameter(const mpm_sim* s) { return s ? s->render_diameter : 0.f; }
void* mpm_posvel_device_ptr(mpm_sim* s) { return s ? s->posvel : nullptr; }

int mpm_download_particles(mpm_sim* s, float* out) {
    if (int rc = check_sim(s)) return rc;
    if (!out && s->n) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(s->device);
    MPM_CUDA(cudaDeviceSynchronize());
    // Particles held in bin order are put back in index order in the spare
    // buffer (no state changes).
    const int c = s->ps.cur;
    const Particles* Psrc = &s->ps.P[c];
    if (!s->ps.canonical) {
        launch_canonicalize(s->ps.P[c], s->ps.id[c], s->ps.P[c ^ 1], nullptr, s->n, nullptr);
        MPM_CUDA(cudaGetLastError());
        MPM_CUDA(cudaDeviceSynchronize());
        Psrc = &s->ps.P[c ^ 1];
    }
    MPM_CUDA(download_records(*Psrc, out, s->n, nullptr, nullptr));
    return MPM_OK;
}

int mpm_download_grid(mpm_sim* s, int32_t* out) {
    if (int rc = check_sim(s)) return rc;
    if (!out && s->grid_count) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(s->device);
    if (int rc = sync_ref_grid(s, nullptr)) return rc;
    MPM_CUDA(cudaDeviceSynchronize());
    if (s->grid_count)
        MPM_CUDA(cudaMemcpy(out, s->grid_ref, sizeof(int4) * (size_t)s->grid_count,
                            cudaMemcpyDeviceToHost));
    return MPM_OK;
}

int mpm_download_posvel(mpm_sim* s, float* out, void* stream) {
    if (int rc = check_sim(s)) return rc;
    if (!out && s->n) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(s->device);
    if (s->n)
        MPM_CUDA(cudaMemcpyAsync(out, s->posvel, sizeof(float4) * 2 * (size_t)s->n,
                                 cudaMemcpyDeviceToHost, static_cast<cudaStream_t>(stream)));
    return MPM_OK;
}

int mpm_download_posvel_async(mpm_sim* s, float* out, void* stream) {
    if (int rc = check_sim(s)) return rc;
    if (!out && s->n) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(s->device);
    if (!s->copy_stream) {
        MPM_CUDA(cudaMalloc(&s->posvel_snap, sizeof(float4) * 2 * (size_t)(s->max_particles > 0 ? s->max_particles : 1)));
        MPM_CUDA(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
        MPM_CUDA(cudaEventCreateWithFlags(&s->snap_taken, cudaEventDisableTiming));
        MPM_CUDA(cudaEventCreateWithFlags(&s->snap_copied, cudaEventDisableTiming));
        MPM_CUDA(cudaEventRecord(s->snap_copied, s->copy_stream));
    }
    if (!s->n) return MPM_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t bytes = sizeof(float4) * 2 * (size_t)s->n;
    // the previous read-back has left the snapshot before it is overwritten
    MPM_CUDA(cudaStreamWaitEvent(st, s->snap_copied, 0));
    MPM_CUDA(cudaMemcpyAsync(s->posvel_snap, s->posvel, bytes, cudaMemcpyDeviceToDevice, st));
    MPM_CUDA(cudaEventRecord(s->snap_taken, st));
    MPM_CUDA(cudaStreamWaitEvent(s->copy_stream, s->snap_taken, 0));
    MPM_CUDA(cudaMemcpyAsync(out, s->posvel_snap, bytes, cudaMemcpyDeviceToHost, s->copy_stream));
    MPM_CUDA(cudaEventRecord(s->snap_copied, s->copy_stream));
    return MPM_OK;
}

int mpm_wait_posvel(mpm_sim* s, void* stream) {
    if (int rc = check_sim(s)) return rc;
    if (!s->snap_copied) return MPM_OK;
    DeviceGuard g(s->device);
    if (stream) MPM_CUDA(cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), s->snap_copied, 0));
    else MPM_CUDA(cudaEventSynchronize(s->snap_copied));
    return MPM_OK;
}

int mpm_dispatch(mpm_sim* s, int kernel, void* stream) {
    if (int rc = check_sim(s)) return rc;
    if (!s->loaded) return fail(MPM_E_STATE, "no scene loaded (call reset first)");
    DeviceGuard g(s->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (kernel < MPM_KERNEL_CLEAR_GRID || kernel > MPM_KERNEL_COPY_POSITION)
        return fail(MPM_E_INVALID, "unknown kernel id");
    const SimConsts k = s->consts();
    if (int rc = sync_ref_grid(s, st)) return rc;
    if (int rc = ensure_canonical(s, st)) return rc;
    sorted_invalidate(s->sorted);
    dispatch_kernel(s, kernel, k, st);
    MPM_CUDA(cudaGetLastError());
    return MPM_OK;
}

int mpm_set_engine(mpm_sim* s, int engine) {
    if (int rc = check_sim(s)) return rc;
    if (engine != MPM_ENGINE_SORTED && engine != MPM_ENGINE_DISPATCH)
        return fail(MPM_E_INVALID, "unknown engine");
    s->engine = engine;
    return MPM_OK;
}

int mpm_get_engine(const mpm_sim* s) { return s ? s->engine : MPM_E_INVALID; }

int mpm_synchronize(mpm_sim* s) {
    if (int rc = check_sim(s)) return rc;
    DeviceGuard g(s->device);
    MPM_CUDA(cudaDeviceSynchronize());
    return MPM_OK;
}

int mpm_check_health(mpm_sim* s, mpm_health* out) {
    if (int rc = check_sim(s)) return rc;
    if (!out) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(s->device);
    MPM_CUDA(cudaDeviceSynchronize());
    MPM_CUDA(cudaMemset(s->counters + 1, 0, sizeof(unsigned long long)));
    launch_count_nonfinite(s->ps.P[s->ps.cur], s->n, s->counters + 1, nullptr);
    unsigned long long h[2] = {0, 0};
    MPM_CUDA(cudaMemcpy(h, s->counters, sizeof(h), cudaMemcpyDeviceToHost));
    out->out_of_range_accesses = (int64_t)h[0];
    out->nonfinite_particles = (int64_t)h[1];
    return h[1] ? fail(MPM_E_NONFINITE, "non-finite particle state") : MPM_OK;
}

int mpm_set_profiling(mpm_sim* s, int enable) {
    if (int rc = check_sim(s)) return rc;
    DeviceGuard g(s->device);
    s->prof.reset();
    s->prof.enabled = enable != 0;
    return MPM_OK;
}

int mpm_kernel_stats(mpm_sim* s, mpm_kernel_stat* out, int max_entries) {
    if (int rc = check_sim(s)) return rc;
    if (max_entries < 0 || (max_entries > 0 && !out)) return fail(MPM_E_INVALID, "bad arguments");
    DeviceGuard g(s->device);
    if (s->prof.collect() != 0) return fail(MPM_E_CUDA, "profiling events failed");
    int count = 0;
    for (int id = 0; id < KID_COUNT; ++id) {
        if (s->prof.launches[id] == 0) continue;
        if (count < max_entries) {
            out[count].name = kernel_name(id);
            out[count].launches = s->prof.launches[id];
            out[count].timed_launches = s->prof.timed[id];
            out[count].total_ms = s->prof.total_ms[id];
        }
        ++count;
    }
    return count;
}

int64_t mpm_launch_count(const mpm_sim* s) {
    if (!s) return 0;
    long long t = 0;
    for (int id = 0; id < KID_COUNT; ++id) t += s->prof.launches[id];
    return t;
}

const char* mpm_error_string(int code) {
    switch (code) {
        case MPM_OK: return "ok";
        case MPM_E_INVALID: return "invalid argument";
        case MPM_E_CAPACITY: return "particle capacity exceeded";
        case MPM_E_GRID_CAPACITY: return "gridCount should be equal to or less than maxGridCount";
        case MPM_E_CUDA: return "CUDA error";
        case MPM_E_NO_DEVICE: return "no CUDA device";
        case MPM_E_STATE: return "no scene loaded";
        case MPM_E_NONFINITE: return "non-finite particle state";
        default: return "unknown error";
    }
}

const char* mpm_last_error(void) { return g_last_error.c_str(); }

int mpm_scene_dambreak(float* out, int max_particles, const double init_box[3], uint64_t seed) {
    if (!out || !init_box || max_particles < 0) return fail(MPM_E_INVALID, "bad arguments");
    return scene_dambreak(out, max_particles, init_box, seed);
}

int mpm_scene_lattice(float* out, int n_per_axis, double origin, double spacing, double jitter,
                      uint64_t seed) {
    if (!out || n_per_axis < 0 || n_per_axis > 1290) return fail(MPM_E_INVALID, "bad arguments");
    return scene_lattice(out, n_per_axis, origin, spacing, jitter, seed);
}

int mpm_probe_conversions(const float* in, int n, float fm, int32_t* enc_out, float* dec_out) {
    if (n < 0 || (n > 0 && (!in || !enc_out || !dec_out))) return fail(MPM_E_INVALID, "bad arguments");
    if (n == 0) return MPM_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MPM_E_NO_DEVICE, "no CUDA device");
    }
    float* d_in = nullptr;
    int* d_enc = nullptr;
    float* d_dec = nullptr;
    cudaError_t e = cudaMalloc(&d_in, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&d_enc, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc(&d_dec, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMemcpy(d_in, in, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_convert_probe(d_in, n, fm, d_enc, d_dec, nullptr);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(enc_out, d_enc, sizeof(int) * n, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(dec_out, d_dec, sizeof(float) * n, cudaMemcpyDeviceToHost);
    cudaFree(d_in);
    cudaFree(d_enc);
    cudaFree(d_dec);
    if (e != cudaSuccess) return cuda_fail(e, "mpm_probe_conversions");
    return MPM_OK;
}

int mpm_probe_packed(const float* a, const float* b, int n, float* out) {
    if (n < 0 || (n % 2) || (n > 0 && (!a || !b || !out))) return fail(MPM_E_INVALID, "bad arguments");
    if (n == 0) return MPM_OK;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MPM_E_NO_DEVICE, "no CUDA device");
    }
    float* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(float) * 8 * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(d, a, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, sizeof(float) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_packed_probe(d, d + n, n / 2, d + 2 * (size_t)n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpy(out, d + 2 * (size_t)n, sizeof(float) * 6 * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "mpm_probe_packed");
    return MPM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches
// ---------------------------------------------------------------------------

struct mpm_batch {
    int device = 0;
    std::vector<mpm_scene_desc> desc;
    std::vector<SimConsts> consts;
    std::vector<long long> first;  // first particle of each scene
    int n = 0;
    ParticleStore ps{};
    float4* posvel = nullptr;
    unsigned long long* counters = nullptr;  // [0] out-of-range, [1] non-finite scratch
    SortedEngine* sorted = nullptr;
    bool graph = true;
    bool stepped = false;
    LaunchProfiler prof;
};

namespace {

int check_batch(const mpm_batch* b) {
    if (!b) return fail(MPM_E_INVALID, "null batch handle");
    return MPM_OK;
}

// SimConsts of one scene; MPM_OK or an error for an unusable description.
int scene_consts(const mpm_scene_desc& d, SimConsts& k) {
    if (d.num_particles < 0) return fail(MPM_E_INVALID, "negative particle count");
    for (int a = 0; a < 3; ++a)
        if (!(d.init_box[a] >= 0.f) || !std::isfinite(d.init_box[a]))
            return fail(MPM_E_INVALID, "init box size must be finite and non-negative");
    const long long gc = grid_count_of(d.init_box);
    if (gc > 0x7fffffffLL) return fail(MPM_E_GRID_CAPACITY, "gridCount exceeds the i32 index range");
    k = SimConsts{};
    k.stiffness = d.stiffness;
    k.rest_density = d.rest_density;
    k.dynamic_viscosity = d.dynamic_viscosity;
    k.dt = d.dt;
    k.fm = d.fixed_point_multiplier;
    for (int a = 0; a < 3; ++a) {
        k.init_box[a] = d.init_box[a];
        k.real_box[a] = d.real_box[a];
        k.gravity[a] = d.gravity[a];
    }
    k.Y = f2i_trunc_sat(d.init_box[1]);
    k.Z = f2i_trunc_sat(d.init_box[2]);
    k.grid_count = (int)gc;
    k.n = d.num_particles;
    if (k.Y <= 0 || k.Z <= 0 || k.grid_count <= 0)
        return fail(MPM_E_INVALID, "batched scenes need a non-degenerate grid");
    return MPM_OK;
}

void free_batch(mpm_batch* b) {
    for (int i = 0; i < 2; ++i) {
        cudaFree(b->ps.P[i].p0);
        cudaFree(b->ps.P[i].p1);
        cudaFree(b->ps.P[i].p2);
        cudaFree(b->ps.P[i].p3);
        cudaFree(b->ps.id[i]);
    }
    cudaFree(b->posvel);
    cudaFree(b->counters);
    if (b->sorted) sorted_destroy(b->sorted);
    b->prof.release();
    delete b;
}

}  // namespace

extern "C" {

int mpm_batch_create(const mpm_scene_desc* scenes, int num_scenes, const float* aos80,
                     mpm_batch** out) {
    if (!out) return fail(MPM_E_INVALID, "out is null");
    *out = nullptr;
    if (!scenes || num_scenes < 1) return fail(MPM_E_INVALID, "a batch needs at least one scene");
    std::vector<SimConsts> ks((size_t)num_scenes);
    std::vector<long long> first((size_t)num_scenes);
    long long n = 0;
    for (int s = 0; s < num_scenes; ++s) {
        if (int rc = scene_consts(scenes[s], ks[(size_t)s])) return rc;
        first[(size_t)s] = n;
        n += scenes[s].num_particles;
    }
    if (n > 0x7fffffffLL / 2) return fail(MPM_E_CAPACITY, "too many particles in the batch");
    if (n > 0 && !aos80) return fail(MPM_E_INVALID, "particle array is null");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(MPM_E_NO_DEVICE, "no CUDA device");
    }
    mpm_batch* b = new (std::nothrow) mpm_batch();
    if (!b) return fail(MPM_E_INVALID, "out of host memory");
    b->desc.assign(scenes, scenes + num_scenes);
    b->consts = ks;
    b->first = first;
    b->n = (int)n;
    MPM_CUDA(cudaGetDevice(&b->device));
    const size_t np = (size_t)(n > 0 ? n : 1);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2; ++i) {
        Particles& P = b->ps.P[i];
        float4** pp[4] = {&P.p0, &P.p1, &P.p2, &P.p3};
        for (int q = 0; q < 4 && e == cudaSuccess; ++q) e = cudaMalloc(pp[q], sizeof(float4) * np);
        if (e == cudaSuccess) e = cudaMalloc(&b->ps.id[i], sizeof(uint32_t) * np);
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->posvel, sizeof(float4) * 2 * np);
    if (e == cudaSuccess) e = cudaMalloc(&b->counters, sizeof(unsigned long long) * 2);
    if (e == cudaSuccess) e = cudaMemset(b->counters, 0, sizeof(unsigned long long) * 2);
    if (e == cudaSuccess) e = cudaMemset(b->posvel, 0, sizeof(float4) * 2 * np);
    if (e == cudaSuccess) e = upload_records(b->ps.P[0], aos80, (int)n, nullptr, nullptr);
    if (e == cudaSuccess) {
        launch_iota(b->ps.id[0], (int)n, nullptr);
        e = cudaGetLastError();
    }
    b->ps.cur = 0;
    b->ps.canonical = true;
    if (e == cudaSuccess && sorted_create(&b->sorted, (int)np) != 0) e = cudaErrorMemoryAllocation;
    if (e == cudaSuccess && sorted_configure_batch(b->sorted, ks.data(), num_scenes) != 0) {
        const std::string msg = std::string("batch: ") + sorted_error();
        free_batch(b);
        return fail(MPM_E_CUDA, msg);
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "mpm_batch_create");
        free_batch(b);
        return rc;
    }
    *out = b;
    return MPM_OK;
}

int mpm_batch_destroy(mpm_batch* b) {
    if (!b) return MPM_OK;
    DeviceGuard g(b->device);
    cudaDeviceSynchronize();
    free_batch(b);
    return MPM_OK;
}

int mpm_batch_num_scenes(const mpm_batch* b) { return b ? (int)b->desc.size() : 0; }
int64_t mpm_batch_num_particles(const mpm_batch* b) { return b ? b->n : 0; }

int mpm_batch_step(mpm_batch* b, int substeps, void* stream) {
    if (int rc = check_batch(b)) return rc;
    if (substeps < 0) return fail(MPM_E_INVALID, "negative substep count");
    if (substeps == 0 || b->n == 0) return MPM_OK;
    DeviceGuard g(b->device);
    if (!g.ok) return fail(MPM_E_CUDA, "cannot select the batch's device");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (sorted_step(b->sorted, &b->ps, b->posvel, b->counters, b->consts[0], substeps, st, &b->prof,
                    b->graph) != 0)
        return fail(MPM_E_CUDA, std::string("batch: ") + sorted_error());
    b->stepped = true;
    MPM_CUDA(cudaGetLastError());
    return MPM_OK;
}

int mpm_batch_upload(mpm_batch* b, const float* aos80) {
    if (int rc = check_batch(b)) return rc;
    if (!aos80 && b->n) return fail(MPM_E_INVALID, "particle array is null");
    DeviceGuard g(b->device);
    if (!g.ok) return fail(MPM_E_CUDA, "cannot select the batch's device");
    MPM_CUDA(cudaDeviceSynchronize());
    b->ps.cur = 0;
    b->ps.canonical = true;
    MPM_CUDA(upload_records(b->ps.P[0], aos80, b->n, nullptr, nullptr));
    launch_iota(b->ps.id[0], b->n, nullptr);
    MPM_CUDA(cudaGetLastError());
    MPM_CUDA(cudaMemset(b->counters, 0, sizeof(unsigned long long) * 2));
    if (b->n) MPM_CUDA(cudaMemset(b->posvel, 0, sizeof(float4) * 2 * (size_t)b->n));
    sorted_invalidate(b->sorted);
    b->stepped = false;
    MPM_CUDA(cudaDeviceSynchronize());
    return MPM_OK;
}

int mpm_batch_set_scene(mpm_batch* b, int scene, const mpm_scene_desc* desc) {
    if (int rc = check_batch(b)) return rc;
    if (!desc || scene < 0 || scene >= (int)b->desc.size()) return fail(MPM_E_INVALID, "bad scene");
    SimConsts k;
    if (int rc = scene_consts(*desc, k)) return rc;
    DeviceGuard g(b->device);
    if (sorted_set_scene_consts(b->sorted, scene, k, nullptr) != 0)
        return fail(MPM_E_INVALID, std::string("batch: ") + sorted_error());
    b->desc[(size_t)scene] = *desc;
    b->consts[(size_t)scene] = k;
    return MPM_OK;
}

int mpm_batch_set_task_size(mpm_batch* b, int cap) {
    if (int rc = check_batch(b)) return rc;
    if (sorted_set_task_cap(b->sorted, cap) != 0) return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_batch_autotune(mpm_batch* b, int substeps, int* chosen_task_size) {
    if (int rc = check_batch(b)) return rc;
    if (substeps < 1) return fail(MPM_E_INVALID, "substeps must be positive");
    DeviceGuard g(b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    auto step = [&](int ns) {
        return sorted_step(b->sorted, &b->ps, b->posvel, b->counters, b->consts[0], ns, nullptr,
                           &b->prof, b->graph);
    };
    const int rc = tune_task_cap(b->sorted, b->ps, b->n, b->posvel, b->counters, substeps, nullptr,
                                 step, chosen_task_size, nullptr);
    b->stepped = false;
    return rc;
}

int mpm_batch_set_graph(mpm_batch* b, int enable) {
    if (int rc = check_batch(b)) return rc;
    b->graph = enable != 0;
    return MPM_OK;
}

int mpm_batch_download_particles(mpm_batch* b, float* out) {
    if (int rc = check_batch(b)) return rc;
    if (!out && b->n) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    const int c = b->ps.cur;
    const Particles* Psrc = &b->ps.P[c];
    if (!b->ps.canonical) {
        launch_canonicalize(b->ps.P[c], b->ps.id[c], b->ps.P[c ^ 1], nullptr, b->n, nullptr);
        MPM_CUDA(cudaGetLastError());
        MPM_CUDA(cudaDeviceSynchronize());
        Psrc = &b->ps.P[c ^ 1];
    }
    MPM_CUDA(download_records(*Psrc, out, b->n, nullptr, nullptr));
    return MPM_OK;
}

int mpm_batch_download_grid(mpm_batch* b, int scene, int32_t* out) {
    if (int rc = check_batch(b)) return rc;
    if (scene < 0 || scene >= (int)b->desc.size()) return fail(MPM_E_INVALID, "bad scene");
    const SimConsts& k = b->consts[(size_t)scene];
    if (!out) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(b->device);
    if (!b->stepped) {
        std::memset(out, 0, sizeof(int32_t) * 4 * (size_t)k.grid_count);
        return MPM_OK;
    }
    int4* tmp = nullptr;
    MPM_CUDA(cudaMalloc(&tmp, sizeof(int4) * (size_t)k.grid_count));
    int rc = MPM_OK;
    if (sorted_export_scene_grid(b->sorted, scene, tmp, nullptr, &b->prof) != 0)
        rc = fail(MPM_E_CUDA, std::string("batch: ") + sorted_error());
    cudaError_t e = rc == MPM_OK ? cudaDeviceSynchronize() : cudaSuccess;
    if (rc == MPM_OK && e == cudaSuccess)
        e = cudaMemcpy(out, tmp, sizeof(int4) * (size_t)k.grid_count, cudaMemcpyDeviceToHost);
    cudaFree(tmp);
    if (rc == MPM_OK && e != cudaSuccess) rc = cuda_fail(e, "mpm_batch_download_grid");
    return rc;
}

void* mpm_batch_posvel_device_ptr(mpm_batch* b) { return b ? b->posvel : nullptr; }

int mpm_batch_check_health(mpm_batch* b, mpm_health* out) {
    if (int rc = check_batch(b)) return rc;
    if (!out) return fail(MPM_E_INVALID, "null output");
    DeviceGuard g(b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    MPM_CUDA(cudaMemset(b->counters + 1, 0, sizeof(unsigned long long)));
    launch_count_nonfinite(b->ps.P[b->ps.cur], b->n, b->counters + 1, nullptr);
    unsigned long long h[2] = {0, 0};
    MPM_CUDA(cudaMemcpy(h, b->counters, sizeof(h), cudaMemcpyDeviceToHost));
    out->out_of_range_accesses = (int64_t)h[0];
    out->nonfinite_particles = (int64_t)h[1];
    return h[1] ? fail(MPM_E_NONFINITE, "non-finite particle state") : MPM_OK;
}

int64_t mpm_batch_launch_count(const mpm_batch* b) {
    if (!b) return 0;
    long long t = 0;
    for (int id = 0; id < KID_COUNT; ++id) t += b->prof.launches[id];
    return t;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiation (forward with checkpoints, backward with recompute)
// ---------------------------------------------------------------------------

struct mpm_adjoint {
    mpm_batch* b = nullptr;
    int max_substeps = 0;
    int every = 1;
    int tape = MPM_TAPE_FP64;
    int T = -1;                      // substeps of the last forward; -1: none
    int nck = 0;                     // checkpoint slots
    // fixed-point tape
    std::vector<Particles> ckpt;     // states after 0, every, 2*every, ..., T substeps
    std::vector<Particles> seg;      // states inside a segment (seg[0] unused)
    int4* gtape = nullptr;           // every x ncells: updated grids of a segment
                                     // (max_substeps x ncells for a full tape)
    // FP64 tape
    std::vector<double*> ckpt64;
    std::vector<double*> seg64;
    double* scratch64[2] = {nullptr, nullptr};
    double4* gtape64 = nullptr;
    // adjoint state
    Particles adj[2]{};
    float4* gadj = nullptr;
    float* stage = nullptr;          // 80 bytes per particle: host records in and out
    AdjScene* scenes_d = nullptr;
    int* pscene_d = nullptr;
    double* pgrad_d = nullptr;
    AdjSort sort;                    // per-substep spatial sort of the adjoint kernels
    std::vector<Particles> seedbuf;  // seeds of mpm_backward, kept between calls
    // The backward as one CUDA graph, captured for (T, every, tape, seed
    // substeps) and replayed while they stay the same.
    cudaGraphExec_t bgraph = nullptr;
    int bg_T = -1, bg_every = 0, bg_tape = -1, bg_cur = 0;
    bool last_taped = false;         // the forward recorded its last segment's tape
    bool bg_last_taped = false;
    std::vector<int> bg_steps;
    int ncells = 0;
    std::vector<int> lbase;
    std::vector<int> bbase;          // first brick of each scene in the sort
};

namespace {

cudaError_t alloc_particles(Particles& P, size_t n) {
    P = Particles{};
    float4** pp[4] = {&P.p0, &P.p1, &P.p2, &P.p3};
    for (int q = 0; q < 4; ++q) {
        const cudaError_t e = cudaMalloc(pp[q], sizeof(float4) * (n ? n : 1));
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

void free_particles(Particles& P) {
    cudaFree(P.p0);
    cudaFree(P.p1);
    cudaFree(P.p2);
    cudaFree(P.p3);
    P = Particles{};
}

cudaError_t copy_particles(const Particles& dst, const Particles& src, int n, cudaStream_t st) {
    const float4* s[4] = {src.p0, src.p1, src.p2, src.p3};
    float4* d[4] = {dst.p0, dst.p1, dst.p2, dst.p3};
    for (int q = 0; q < 4; ++q) {
        const cudaError_t e = cudaMemcpyAsync(d[q], s[q], sizeof(float4) * (size_t)n,
                                              cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// The same for the FP64 tape's records (kRec64 doubles).
cudaError_t upload_records64(double* dst, const float* host, int n, float* stage, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(stage, host, (size_t)80 * (size_t)n, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        launch_records_to_rec64(stage, dst, n, st);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t download_records64(const double* src, float* host, int n, float* stage,
                               cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    launch_rec64_to_records(src, stage, n, st);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(host, stage, (size_t)80 * (size_t)n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

// Puts a canonical state into the batch's particle store and forgets the
// sorted engine's carried state.
cudaError_t batch_load_device(mpm_batch* b, const Particles& src, cudaStream_t st) {
    b->ps.cur = 0;
    b->ps.canonical = true;
    cudaError_t e = copy_particles(b->ps.P[0], src, b->n, st);
    if (e != cudaSuccess) return e;
    launch_iota(b->ps.id[0], b->n, st);
    sorted_invalidate(b->sorted);
    b->stepped = false;
    return cudaGetLastError();
}

// The batch's current state, in particle order, into dst.
void batch_canonical_to(mpm_batch* b, const Particles& dst, cudaStream_t st) {
    const int c = b->ps.cur;
    if (b->ps.canonical) {
        copy_particles(dst, b->ps.P[c], b->n, st);
        return;
    }
    launch_canonicalize(b->ps.P[c], b->ps.id[c], dst, nullptr, b->n, st);
}

void free_tapes(mpm_adjoint* a) {
    for (Particles& P : a->ckpt) free_particles(P);
    for (Particles& P : a->seg) free_particles(P);
    a->ckpt.clear();
    a->seg.clear();
    cudaFree(a->gtape);
    a->gtape = nullptr;
    for (double* p : a->ckpt64) cudaFree(p);
    for (double* p : a->seg64) cudaFree(p);
    a->ckpt64.clear();
    a->seg64.clear();
    for (double*& p : a->scratch64) {
        cudaFree(p);
        p = nullptr;
    }
    cudaFree(a->gtape64);
    a->gtape64 = nullptr;
}

// checkpoint_every == 1 keeps every substep's state and updated grid (a full
// tape): the backward then recomputes nothing.
bool full_tape(const mpm_adjoint* a) { return a->every == 1; }
int tape_grids(const mpm_adjoint* a) { return full_tape(a) ? a->max_substeps : a->every; }

// Allocates the buffers of the selected tape (and frees the other's).
cudaError_t alloc_tape(mpm_adjoint* a) {
    free_tapes(a);
    const size_t np = (size_t)(a->b->n > 0 ? a->b->n : 1);
    const size_t nc = (size_t)a->ncells;
    cudaError_t e = cudaSuccess;
    if (a->tape == MPM_TAPE_FIXED_POINT) {
        a->ckpt.resize((size_t)a->nck);
        for (int i = 0; i < a->nck && e == cudaSuccess; ++i) e = alloc_particles(a->ckpt[(size_t)i], np);
        a->seg.resize((size_t)a->every);
        for (int i = 1; i < a->every && e == cudaSuccess; ++i)
            e = alloc_particles(a->seg[(size_t)i], np);
        if (e == cudaSuccess) e = cudaMalloc(&a->gtape, sizeof(int4) * (size_t)tape_grids(a) * nc);
    } else {
        a->ckpt64.assign((size_t)a->nck, nullptr);
        for (int i = 0; i < a->nck && e == cudaSuccess; ++i)
            e = cudaMalloc(&a->ckpt64[(size_t)i], sizeof(double) * kRec64 * np);
        a->seg64.assign((size_t)a->every, nullptr);
        for (int i = 1; i < a->every && e == cudaSuccess; ++i)
            e = cudaMalloc(&a->seg64[(size_t)i], sizeof(double) * kRec64 * np);
        for (int i = 0; i < 2 && e == cudaSuccess; ++i)
            e = cudaMalloc(&a->scratch64[i], sizeof(double) * kRec64 * np);
        if (e == cudaSuccess)
            e = cudaMalloc(&a->gtape64, sizeof(double4) * (size_t)tape_grids(a) * nc);
    }
    return e;
}

void drop_backward_graph(mpm_adjoint* a) {
    if (a->bgraph) cudaGraphExecDestroy(a->bgraph);
    a->bgraph = nullptr;
    a->bg_T = -1;
}

void free_adjoint(mpm_adjoint* a) {
    drop_backward_graph(a);
    for (Particles& P : a->seedbuf) free_particles(P);
    free_tapes(a);
    free_particles(a->adj[0]);
    free_particles(a->adj[1]);
    cudaFree(a->gadj);
    cudaFree(a->stage);
    cudaFree(a->scenes_d);
    cudaFree(a->pscene_d);
    cudaFree(a->pgrad_d);
    cudaFree(a->sort.key_rank);
    cudaFree(a->sort.perm);
    cudaFree(a->sort.bin_count);
    cudaFree(a->sort.bin_first);
    cudaFree(a->sort.placed);
    if (a->b) mpm_batch_destroy(a->b);
    delete a;
}

int upload_adj_scenes(mpm_adjoint* a) {
    const int S = (int)a->b->consts.size();
    std::vector<AdjScene> hs((size_t)S);
    for (int s = 0; s < S; ++s) {
        AdjScene& h = hs[(size_t)s];
        h.k = a->b->consts[(size_t)s];
        h.lbase = a->lbase[(size_t)s];
        h.bbase = a->bbase[(size_t)s];
        int BX = 0;
        adj_bricks(h.k, BX, h.BY, h.BZ);
    }
    MPM_CUDA(cudaMemcpy(a->scenes_d, hs.data(), sizeof(AdjScene) * (size_t)S, cudaMemcpyHostToDevice));
    return MPM_OK;
}

// Threads per particle in the adjoint kernels: three (one per stencil
// x-slab) while one thread per particle would leave most of the GPU idle
// (fewer particles than 512 per SM), else one.
int adj_lanes(long long n) {
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm < 1)
        nsm = 1;
    return n < 512LL * nsm ? 3 : 1;
}

// The whole backward of the last forward, enqueued on `st` (kernels,
// memsets and device copies only, so it can be captured): for each
// checkpoint segment from the last, recompute its states and updated grids
// (unless the full tape kept them), then run its adjoint substeps in reverse,
// adding the seeds at their substeps.  *cur_out: the adjoint buffer that
// ends up holding dL/dS_0.
int enqueue_backward(mpm_adjoint* a, const int* seed_steps, int nseeds, cudaStream_t st,
                     int* cur_out) {
    mpm_batch* b = a->b;
    const int n = b->n, S = (int)b->consts.size();
    const bool f64 = a->tape == MPM_TAPE_FP64;
    auto add_seeds = [&](int step, const Particles& A) {
        for (int i = 0; i < nseeds; ++i)
            if (seed_steps[i] == step) launch_particles_axpy(A, a->seedbuf[(size_t)i], n, st);
    };
    int cur = 0;
    float4* z[4] = {a->adj[0].p0, a->adj[0].p1, a->adj[0].p2, a->adj[0].p3};
    for (int q = 0; q < 4; ++q) MPM_CUDA(cudaMemsetAsync(z[q], 0, sizeof(float4) * (size_t)n, st));
    MPM_CUDA(cudaMemsetAsync(a->pgrad_d, 0, sizeof(double) * 2 * (size_t)S, st));
    add_seeds(a->T, a->adj[cur]);
    const int nseg = (a->T + a->every - 1) / a->every;
    const size_t nc = (size_t)a->ncells;
    for (int j = nseg - 1; j >= 0; --j) {
        const int t0 = j * a->every;
        const int t1 = t0 + a->every < a->T ? t0 + a->every : a->T;
        // recompute the segment: states and updated grids of every substep
        // (a full tape kept them all)
        const size_t g0 = full_tape(a) ? (size_t)t0 : 0;  // tape grid of substep t0
        if (full_tape(a) || (a->last_taped && j == nseg - 1)) {
        } else if (f64) {
            const double* curS = a->ckpt64[(size_t)j];
            for (int t = t0; t < t1; ++t) {
                double* dst = t + 1 < t1 ? a->seg64[(size_t)(t + 1 - t0)] : a->scratch64[0];
                launch_substep64(curS, a->gtape64 + (size_t)(t - t0) * nc, dst, a->scenes_d, S,
                                 a->pscene_d, n, a->ncells, st);
                curS = dst;
            }
        } else {
            if (cudaError_t e = batch_load_device(b, a->ckpt[(size_t)j], st); e != cudaSuccess)
                return cuda_fail(e, "mpm_backward recompute");
            for (int t = t0; t < t1; ++t) {
                if (sorted_step(b->sorted, &b->ps, b->posvel, b->counters, b->consts[0], 1, st,
                                &b->prof, b->graph) != 0)
                    return fail(MPM_E_CUDA, std::string("backward recompute: ") + sorted_error());
                b->stepped = true;
                // the updated grid, and the state after the substep when the
                // segment goes on, in one launch
                int4* gt = a->gtape + (size_t)(t - t0) * nc;
                const int rc = t + 1 < t1
                                   ? sorted_export_all_canonical(b->sorted, gt, b->ps,
                                                                 a->seg[(size_t)(t + 1 - t0)], n, st,
                                                                 &b->prof)
                                   : sorted_export_all(b->sorted, gt, st, &b->prof);
                if (rc != 0)
                    return fail(MPM_E_CUDA, std::string("backward recompute: ") + sorted_error());
            }
        }
        // adjoint substeps in reverse
        for (int t = t1 - 1; t >= t0; --t) {
            if (f64) {
                const double* Sx = t == t0 ? a->ckpt64[(size_t)j] : a->seg64[(size_t)(t - t0)];
                launch_adjoint_substep64(Sx, a->gtape64 + (g0 + (size_t)(t - t0)) * nc, a->adj[cur],
                                         a->adj[cur ^ 1], a->gadj, a->scenes_d, S, a->pscene_d, n,
                                         a->ncells, a->pgrad_d, a->sort, st);
            } else {
                const Particles& Sx = t == t0 ? a->ckpt[(size_t)j] : a->seg[(size_t)(t - t0)];
                launch_adjoint_substep(Sx, a->gtape + (g0 + (size_t)(t - t0)) * nc, a->adj[cur],
                                       a->adj[cur ^ 1], a->gadj, a->scenes_d, S, a->pscene_d, n,
                                       a->ncells, a->pgrad_d, a->sort, st);
            }
            cur ^= 1;
            add_seeds(t, a->adj[cur]);
        }
    }
    MPM_CUDA(cudaGetLastError());
    *cur_out = cur;
    return MPM_OK;
}

// Checkpoint slot of the state after `step` substeps of a T-substep forward
// (-1: not kept).
int ckpt_slot(const mpm_adjoint* a, int step, int T) {
    if (step == T) return (T + a->every - 1) / a->every;
    if (step >= 0 && step < T && step % a->every == 0) return step / a->every;
    return -1;
}

}  // namespace

extern "C" {

int mpm_adjoint_create(const mpm_scene_desc* scenes, int num_scenes, int max_substeps,
                       int checkpoint_every, mpm_adjoint** out) {
    if (!out) return fail(MPM_E_INVALID, "out is null");
    *out = nullptr;
    if (max_substeps < 1 || checkpoint_every < 1)
        return fail(MPM_E_INVALID, "max_substeps and checkpoint_every must be positive");
    if (!scenes || num_scenes < 1) return fail(MPM_E_INVALID, "a batch needs at least one scene");
    long long n = 0, cells = 0;
    long long bricks = 0;
    std::vector<int> lbase((size_t)num_scenes), bbase((size_t)num_scenes);
    std::vector<int> pscene;
    for (int s = 0; s < num_scenes; ++s) {
        SimConsts k;
        if (int rc = scene_consts(scenes[s], k)) return rc;
        lbase[(size_t)s] = (int)cells;
        bbase[(size_t)s] = (int)bricks;
        cells += k.grid_count;
        int BX = 0, BY = 0, BZ = 0;
        adj_bricks(k, BX, BY, BZ);
        bricks += (long long)BX * BY * BZ;
        if (bricks > 0x3fffffffLL) return fail(MPM_E_CAPACITY, "batch too large");
        n += scenes[s].num_particles;
        if (cells > 0x7fffffffLL || n > 0x3fffffffLL) return fail(MPM_E_CAPACITY, "batch too large");
        pscene.insert(pscene.end(), (size_t)scenes[s].num_particles, s);
    }
    // the engine starts from zeros; mpm_forward_ckpt loads the real state
    std::vector<float> zeros((size_t)20 * (size_t)(n > 0 ? n : 1), 0.0f);
    mpm_batch* b = nullptr;
    if (int rc = mpm_batch_create(scenes, num_scenes, zeros.data(), &b)) return rc;
    mpm_adjoint* a = new (std::nothrow) mpm_adjoint();
    if (!a) {
        mpm_batch_destroy(b);
        return fail(MPM_E_INVALID, "out of host memory");
    }
    a->b = b;
    a->max_substeps = max_substeps;
    a->every = checkpoint_every < max_substeps ? checkpoint_every : max_substeps;
    a->nck = (max_substeps + a->every - 1) / a->every + 1;
    a->ncells = (int)cells;
    a->lbase = lbase;
    a->bbase = bbase;
    DeviceGuard g(b->device);
    const size_t np = (size_t)(n > 0 ? n : 1);
    AdjSort& so = a->sort;
    so.nbins = (int)bricks + 1;
    so.lanes = adj_lanes(n);
    cudaError_t e = alloc_tape(a);
    if (e == cudaSuccess) e = cudaMalloc(&so.key_rank, sizeof(int2) * np);
    if (e == cudaSuccess) e = cudaMalloc(&so.perm, sizeof(int) * np);
    if (e == cudaSuccess) e = cudaMalloc(&so.bin_count, sizeof(int) * (size_t)so.nbins);
    if (e == cudaSuccess) e = cudaMalloc(&so.bin_first, sizeof(int) * (size_t)so.nbins);
    if (e == cudaSuccess) e = cudaMalloc(&so.placed, sizeof(int));
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = alloc_particles(a->adj[i], np);
    if (e == cudaSuccess) e = cudaMalloc(&a->gadj, sizeof(float4) * (size_t)cells);
    if (e == cudaSuccess) e = cudaMalloc(&a->stage, (size_t)80 * np);
    if (e == cudaSuccess) e = cudaMalloc(&a->scenes_d, sizeof(AdjScene) * (size_t)num_scenes);
    if (e == cudaSuccess) e = cudaMalloc(&a->pscene_d, sizeof(int) * np);
    if (e == cudaSuccess) e = cudaMalloc(&a->pgrad_d, sizeof(double) * 2 * (size_t)num_scenes);
    if (e == cudaSuccess && n)
        e = cudaMemcpy(a->pscene_d, pscene.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        const int rc = cuda_fail(e, "mpm_adjoint_create");
        free_adjoint(a);
        return rc;
    }
    if (int rc = upload_adj_scenes(a)) {
        free_adjoint(a);
        return rc;
    }
    *out = a;
    return MPM_OK;
}

int mpm_adjoint_destroy(mpm_adjoint* a) {
    if (!a) return MPM_OK;
    DeviceGuard g(a->b->device);
    cudaDeviceSynchronize();
    free_adjoint(a);
    return MPM_OK;
}

int mpm_adjoint_set_tape(mpm_adjoint* a, int tape) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (tape != MPM_TAPE_FIXED_POINT && tape != MPM_TAPE_FP64) return fail(MPM_E_INVALID, "unknown tape");
    if (tape == a->tape) return MPM_OK;
    DeviceGuard g(a->b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    a->tape = tape;
    a->T = -1;
    drop_backward_graph(a);  // it holds the old tape's buffers
    MPM_CUDA(alloc_tape(a));
    return MPM_OK;
}

int mpm_adjoint_set_scene(mpm_adjoint* a, int scene, const mpm_scene_desc* desc) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (int rc = mpm_batch_set_scene(a->b, scene, desc)) return rc;
    DeviceGuard g(a->b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    a->T = -1;
    return upload_adj_scenes(a);
}

int mpm_forward_ckpt(mpm_adjoint* a, const float* init, int substeps, void* stream) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    mpm_batch* b = a->b;
    if (substeps < 0 || substeps > a->max_substeps)
        return fail(MPM_E_INVALID, "substeps outside [0, max_substeps]");
    if (!init && b->n) return fail(MPM_E_INVALID, "initial state is null");
    DeviceGuard g(b->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = b->n, S = (int)b->consts.size();
    a->T = -1;
    MPM_CUDA(cudaStreamSynchronize(st));
    // The last checkpoint segment is the first one the backward needs: its
    // states and updated grids are recorded here, as the backward's
    // recompute would record them, so that it is not recomputed.
    const int nseg = (substeps + a->every - 1) / a->every;
    const int last_t0 = nseg > 0 ? (nseg - 1) * a->every : 0;
    const bool tape_last = !full_tape(a) && substeps > 0;
    const size_t nc = (size_t)a->ncells;
    if (a->tape == MPM_TAPE_FP64) {
        MPM_CUDA(upload_records64(a->ckpt64[0], init, n, a->stage, st));
        const double* cur = a->ckpt64[0];
        for (int t = 0; t < substeps; ++t) {
            const int slot = ckpt_slot(a, t + 1, substeps);
            double* dst = slot >= 0 ? a->ckpt64[(size_t)slot] : a->scratch64[t & 1];
            double4* G = a->gtape64 + (full_tape(a) ? (size_t)t * nc : 0);
            if (tape_last && t >= last_t0) {
                G = a->gtape64 + (size_t)(t - last_t0) * nc;
                if (t + 1 < substeps) dst = a->seg64[(size_t)(t + 1 - last_t0)];
            }
            launch_substep64(cur, G, dst, a->scenes_d, S, a->pscene_d, n, a->ncells, st);
            cur = dst;
        }
    } else {
        MPM_CUDA(upload_records(a->ckpt[0], init, n, a->stage, st));
        MPM_CUDA(batch_load_device(b, a->ckpt[0], st));
        int t = 0;
        while (t < substeps) {
            if (tape_last && t >= last_t0) {  // one substep at a time, recording
                if (sorted_step(b->sorted, &b->ps, b->posvel, b->counters, b->consts[0], 1, st,
                                &b->prof, b->graph) != 0)
                    return fail(MPM_E_CUDA, std::string("forward: ") + sorted_error());
                b->stepped = true;
                int4* gt = a->gtape + (size_t)(t - last_t0) * nc;
                ++t;
                const Particles& dst = t < substeps ? a->seg[(size_t)(t - last_t0)]
                                                    : a->ckpt[(size_t)ckpt_slot(a, t, substeps)];
                if (sorted_export_all_canonical(b->sorted, gt, b->ps, dst, n, st, &b->prof) != 0)
                    return fail(MPM_E_CUDA, std::string("forward: ") + sorted_error());
                continue;
            }
            const int ns = substeps - t < a->every ? substeps - t : a->every;
            if (sorted_step(b->sorted, &b->ps, b->posvel, b->counters, b->consts[0], ns, st,
                            &b->prof, b->graph) != 0)
                return fail(MPM_E_CUDA, std::string("forward: ") + sorted_error());
            b->stepped = true;
            const Particles& dst = a->ckpt[(size_t)ckpt_slot(a, t + ns, substeps)];
            if (full_tape(a)) {
                if (sorted_export_all_canonical(b->sorted, a->gtape + (size_t)t * (size_t)a->ncells,
                                                b->ps, dst, n, st, &b->prof) != 0)
                    return fail(MPM_E_CUDA, std::string("forward: ") + sorted_error());
            } else {
                batch_canonical_to(b, dst, st);
            }
            t += ns;
        }
    }
    MPM_CUDA(cudaGetLastError());
    a->T = substeps;
    a->last_taped = tape_last;
    return MPM_OK;
}

int mpm_adjoint_state(mpm_adjoint* a, int substep, float* out) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (a->T < 0) return fail(MPM_E_STATE, "no forward run");
    if (!out && a->b->n) return fail(MPM_E_INVALID, "null output");
    const int j = ckpt_slot(a, substep, a->T);
    if (j < 0) return fail(MPM_E_INVALID, "substep is not a checkpoint");
    DeviceGuard g(a->b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    if (a->tape == MPM_TAPE_FP64) MPM_CUDA(download_records64(a->ckpt64[(size_t)j], out, a->b->n, a->stage, nullptr));
    else MPM_CUDA(download_records(a->ckpt[(size_t)j], out, a->b->n, a->stage, nullptr));
    return MPM_OK;
}

int mpm_backward(mpm_adjoint* a, const float* seeds, const int* seed_steps, int nseeds,
                 float* grad_init, double* grad_params, void* stream) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (nseeds < 0 || (nseeds > 0 && (!seeds || !seed_steps)))
        return fail(MPM_E_INVALID, "bad seeds");
    std::vector<const float*> list((size_t)(nseeds > 0 ? nseeds : 1));
    for (int i = 0; i < nseeds; ++i) list[(size_t)i] = seeds + (size_t)i * 20 * (size_t)a->b->n;
    return mpm_backward_list(a, list.data(), seed_steps, nseeds, grad_init, grad_params, stream);
}

int mpm_backward_list(mpm_adjoint* a, const float* const* seeds, const int* seed_steps, int nseeds,
                      float* grad_init, double* grad_params, void* stream) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    mpm_batch* b = a->b;
    if (a->T < 0) return fail(MPM_E_STATE, "no forward run");
    if (nseeds < 0 || (nseeds > 0 && (!seeds || !seed_steps)))
        return fail(MPM_E_INVALID, "bad seeds");
    for (int i = 0; i < nseeds; ++i)
        if (!seeds[i] && b->n) return fail(MPM_E_INVALID, "null seed block");
    for (int i = 0; i < nseeds; ++i)
        if (seed_steps[i] < 0 || seed_steps[i] > a->T)
            return fail(MPM_E_INVALID, "seed substep outside [0, T]");
    DeviceGuard g(b->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = b->n, S = (int)b->consts.size();
    MPM_CUDA(cudaStreamSynchronize(st));
    // seeds into device streams kept between calls (a captured backward
    // reads them at fixed addresses)
    while ((int)a->seedbuf.size() < nseeds) {
        drop_backward_graph(a);
        Particles P{};
        const cudaError_t e = alloc_particles(P, (size_t)(n > 0 ? n : 1));
        if (e != cudaSuccess) {
            free_particles(P);
            return cuda_fail(e, "mpm_backward seeds");
        }
        a->seedbuf.push_back(P);
    }
    for (int i = 0; i < nseeds; ++i)
        MPM_CUDA(upload_records(a->seedbuf[(size_t)i], seeds[i], n, a->stage, st));
    const std::vector<int> steps(seed_steps, seed_steps + nseeds);
    int cur = 0;
    if (b->prof.enabled) {  // per-launch profiling: no graph
        if (int rc = enqueue_backward(a, seed_steps, nseeds, st, &cur)) return rc;
    } else if (a->bgraph && a->bg_T == a->T && a->bg_every == a->every && a->bg_tape == a->tape &&
               a->bg_last_taped == a->last_taped && a->bg_steps == steps) {
        MPM_CUDA(cudaGraphLaunch(a->bgraph, st));
        cur = a->bg_cur;
    } else {
        drop_backward_graph(a);
        cudaStream_t cs = nullptr;
        MPM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        const bool engine_graph = b->graph;
        b->graph = false;  // the engine's kernels go straight into this graph
        cudaGraph_t graph = nullptr;
        int rc = 0;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = enqueue_backward(a, seed_steps, nseeds, cs, &cur);
            e = cudaStreamEndCapture(cs, &graph);
        }
        b->graph = engine_graph;
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess && rc == 0) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        if (rc) return rc;
        if (e != cudaSuccess) return cuda_fail(e, "mpm_backward capture");
        a->bgraph = exec;
        a->bg_T = a->T;
        a->bg_every = a->every;
        a->bg_tape = a->tape;
        a->bg_last_taped = a->last_taped;
        a->bg_steps = steps;
        a->bg_cur = cur;
        MPM_CUDA(cudaGraphLaunch(exec, st));
    }
    // the recompute of the earlier segments reused the buffers that held the
    // forward's record of the last one: a further backward recomputes it
    a->last_taped = false;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "mpm_backward");
    if (grad_init) MPM_CUDA(download_records(a->adj[cur], grad_init, n, a->stage, st));
    if (grad_params)
        MPM_CUDA(cudaMemcpy(grad_params, a->pgrad_d, sizeof(double) * 2 * (size_t)S,
                            cudaMemcpyDeviceToHost));
    return MPM_OK;
}

}  // extern "C"
