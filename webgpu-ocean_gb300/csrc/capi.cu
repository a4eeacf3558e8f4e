// capi.cu -- the C ABI of libmpm.so (include/mpm.h): simulator handle,
// device memory, scene builders and the per-frame stage sequencing of
// MLSMPMSimulator (mls-mpm/mls-mpm.ts:12-276).  Batches are in
// capi_batch.cu, differentiation in capi_adjoint.cu.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace mpm;

namespace {

thread_local std::string g_last_error;

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

}  // namespace

namespace mpm {
// Lets other translation units report a message through mpm_last_error().
void set_last_error(const std::string& msg) { g_last_error = msg; }

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

// mls-mpm.ts:229 gridCount = ceil(X) * ceil(Y) * ceil(Z)
long long grid_count_of(const float b[3]) {
    return (long long)std::ceil((double)b[0]) * (long long)std::ceil((double)b[1]) *
           (long long)std::ceil((double)b[2]);
}

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

int mpm_set_lane_table_min(mpm_sim* s, int min_particles) {
    if (int rc = check_sim(s)) return rc;
    if (sorted_set_lane_table_min(s->sorted, min_particles) != 0)
        return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_get_lane_table_min(const mpm_sim* s) {
    return s ? sorted_lane_table_min(s->sorted) : MPM_E_INVALID;
}

int mpm_set_task_threads(mpm_sim* s, int threads) {
    if (int rc = check_sim(s)) return rc;
    if (sorted_set_threads(s->sorted, threads) != 0) return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_get_task_threads(const mpm_sim* s) {
    return s ? sorted_threads(s->sorted) : MPM_E_INVALID;
}

int mpm_set_bin_pairing(mpm_sim* s, int max_particles) {
    if (int rc = check_sim(s)) return rc;
    if (sorted_set_pair_max(s->sorted, max_particles) != 0) return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_get_bin_pairing(const mpm_sim* s) {
    return s ? sorted_pair_max(s->sorted) : MPM_E_INVALID;
}


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
    const int rc = tune_engine(s->sorted, s->ps, s->n, s->posvel, s->counters, substeps,
                               s->internal, step, chosen_task_size, nullptr, nullptr);
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
        // Made into locals and committed together, so a failure part-way
        // leaves the handle as it was (and frees what was made).
        float4* snap = nullptr;
        cudaStream_t cs = nullptr;
        cudaEvent_t taken = nullptr, copied = nullptr;
        cudaError_t e = cudaMalloc(&snap, sizeof(float4) * 2 *
                                              (size_t)(s->max_particles > 0 ? s->max_particles : 1));
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&taken, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(copied, cs);
        if (e != cudaSuccess) {
            if (copied) cudaEventDestroy(copied);
            if (taken) cudaEventDestroy(taken);
            if (cs) cudaStreamDestroy(cs);
            cudaFree(snap);
            return cuda_fail(e, "mpm_download_posvel_async set-up");
        }
        s->posvel_snap = snap;
        s->copy_stream = cs;
        s->snap_taken = taken;
        s->snap_copied = copied;
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

