// capi_batch.cu -- the C ABI's batches (mpm_batch_*): many independent
// scenes advanced together by the sorted engine, one launch per stage.
#include "capi_internal.h"

#include <new>

using namespace mpm;

// ---------------------------------------------------------------------------
// Batches
// ---------------------------------------------------------------------------

namespace mpm {

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

}  // namespace mpm

namespace {

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

int mpm_batch_get_task_size(const mpm_batch* b) {
    return b && b->sorted ? sorted_task_cap(b->sorted) : MPM_E_INVALID;
}

int mpm_batch_set_lane_table_min(mpm_batch* b, int min_particles) {
    if (int rc = check_batch(b)) return rc;
    if (sorted_set_lane_table_min(b->sorted, min_particles) != 0)
        return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_batch_get_lane_table_min(const mpm_batch* b) {
    return b && b->sorted ? sorted_lane_table_min(b->sorted) : MPM_E_INVALID;
}

int mpm_batch_set_task_threads(mpm_batch* b, int threads) {
    if (int rc = check_batch(b)) return rc;
    if (sorted_set_threads(b->sorted, threads) != 0) return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_batch_get_task_threads(const mpm_batch* b) {
    return b && b->sorted ? sorted_threads(b->sorted) : MPM_E_INVALID;
}

int mpm_batch_set_bin_pairing(mpm_batch* b, int max_particles) {
    if (int rc = check_batch(b)) return rc;
    if (sorted_set_pair_max(b->sorted, max_particles) != 0) return fail(MPM_E_INVALID, sorted_error());
    return MPM_OK;
}

int mpm_batch_get_bin_pairing(const mpm_batch* b) {
    return b && b->sorted ? sorted_pair_max(b->sorted) : MPM_E_INVALID;
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
    const int rc = tune_engine(b->sorted, b->ps, b->n, b->posvel, b->counters, substeps, nullptr,
                               step, chosen_task_size, nullptr, nullptr);
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

int mpm_batch_set_profiling(mpm_batch* b, int enable) {
    if (int rc = check_batch(b)) return rc;
    DeviceGuard g(b->device);
    b->prof.reset();
    b->prof.enabled = enable != 0;
    return MPM_OK;
}

int mpm_batch_kernel_stats(mpm_batch* b, mpm_kernel_stat* out, int max_entries) {
    if (int rc = check_batch(b)) return rc;
    if (max_entries < 0 || (max_entries > 0 && !out)) return fail(MPM_E_INVALID, "bad arguments");
    DeviceGuard g(b->device);
    if (b->prof.collect() != 0) return fail(MPM_E_CUDA, "profiling events failed");
    int count = 0;
    for (int id = 0; id < KID_COUNT; ++id) {
        if (b->prof.launches[id] == 0) continue;
        if (count < max_entries) {
            out[count].name = kernel_name(id);
            out[count].launches = b->prof.launches[id];
            out[count].timed_launches = b->prof.timed[id];
            out[count].total_ms = b->prof.total_ms[id];
        }
        ++count;
    }
    return count;
}

}  // extern "C"

