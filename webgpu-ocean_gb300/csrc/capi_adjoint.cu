// capi_adjoint.cu -- the C ABI's differentiation (mpm_adjoint_*,
// mpm_forward_ckpt, mpm_backward): batched forward with checkpoints and the
// reverse-mode backward with recompute (adjoint.cu holds the kernels).
#include "capi_internal.h"

#include <new>

#include "adjoint.h"

using namespace mpm;

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
    std::vector<Particles> seg[2];   // states inside a segment (seg[.][0] unused)
    int4* gtape[2] = {nullptr, nullptr};  // every x ncells: updated grids of a segment
                                          // (max_substeps x ncells for a full tape)
    // Segment tape sets: two when a backward can have more than one segment,
    // so that the recompute of segment j - 1 fills one while the adjoint of
    // segment j reads the other.  Segment j of a T-substep run uses set
    // tape_set(a, j); the forward records its last segment in set 0.
    int sets = 1;
    // FP64 tape
    std::vector<double*> ckpt64;
    std::vector<double*> seg64[2];
    double* scratch64[2] = {nullptr, nullptr};
    double4* gtape64[2] = {nullptr, nullptr};
    // adjoint state
    Particles adj[2]{};
    float4* gadj = nullptr;
    float* stage = nullptr;          // 80 bytes per particle: host records in and out
    AdjScene* scenes_d = nullptr;
    int* pscene_d = nullptr;
    double* pgrad_d = nullptr;
    AdjSort sort;                    // per-substep spatial sort of the adjoint kernels
    std::vector<Particles> seedbuf;  // seeds of mpm_backward, kept between calls
    // observation loss (mpm_adjoint_set_observations)
    std::vector<float4*> obs;        // observed positions (n float4 each)
    std::vector<int> obs_steps;      // their substeps
    float* obs_scale = nullptr;      // per scene: f32(2 / its particle count)
    double* obs_loss = nullptr;      // per scene: sum of |x - obs|^2
    bool obs_seeded = false;         // seedbuf[0 .. obs) hold the seeds of the last forward
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
    a->ckpt.clear();
    for (double* p : a->ckpt64) cudaFree(p);
    a->ckpt64.clear();
    for (int k = 0; k < 2; ++k) {
        for (Particles& P : a->seg[k]) free_particles(P);
        a->seg[k].clear();
        cudaFree(a->gtape[k]);
        a->gtape[k] = nullptr;
        for (double* p : a->seg64[k]) cudaFree(p);
        a->seg64[k].clear();
        cudaFree(a->gtape64[k]);
        a->gtape64[k] = nullptr;
        cudaFree(a->scratch64[k]);
        a->scratch64[k] = nullptr;
    }
}

// checkpoint_every == 1 keeps every substep's state and updated grid (a full
// tape): the backward then recomputes nothing.
bool full_tape(const mpm_adjoint* a) { return a->every == 1; }
int tape_grids(const mpm_adjoint* a) { return full_tape(a) ? a->max_substeps : a->every; }
// The segment tape set of segment j of a forward of T substeps: the last
// segment uses set 0 (the forward's record), the ones before it alternate.
int tape_set(const mpm_adjoint* a, int j) {
    const int nseg = (a->T + a->every - 1) / a->every;
    return (nseg - 1 - j) & (a->sets - 1);
}

// Allocates the buffers of the selected tape (and frees the other's).
cudaError_t alloc_tape(mpm_adjoint* a) {
    free_tapes(a);
    const size_t np = (size_t)(a->b->n > 0 ? a->b->n : 1);
    const size_t nc = (size_t)a->ncells;
    a->sets = !full_tape(a) && a->max_substeps > a->every ? 2 : 1;
    cudaError_t e = cudaSuccess;
    if (a->tape == MPM_TAPE_FIXED_POINT) {
        a->ckpt.resize((size_t)a->nck);
        for (int i = 0; i < a->nck && e == cudaSuccess; ++i) e = alloc_particles(a->ckpt[(size_t)i], np);
        for (int k = 0; k < a->sets && e == cudaSuccess; ++k) {
            a->seg[k].resize((size_t)a->every);
            for (int i = 1; i < a->every && e == cudaSuccess; ++i)
                e = alloc_particles(a->seg[k][(size_t)i], np);
            if (e == cudaSuccess)
                e = cudaMalloc(&a->gtape[k], sizeof(int4) * (size_t)tape_grids(a) * nc);
        }
    } else {
        a->ckpt64.assign((size_t)a->nck, nullptr);
        for (int i = 0; i < a->nck && e == cudaSuccess; ++i)
            e = cudaMalloc(&a->ckpt64[(size_t)i], sizeof(double) * kRec64 * np);
        for (int k = 0; k < a->sets && e == cudaSuccess; ++k) {
            a->seg64[k].assign((size_t)a->every, nullptr);
            for (int i = 1; i < a->every && e == cudaSuccess; ++i)
                e = cudaMalloc(&a->seg64[k][(size_t)i], sizeof(double) * kRec64 * np);
            if (e == cudaSuccess)
                e = cudaMalloc(&a->gtape64[k], sizeof(double4) * (size_t)tape_grids(a) * nc);
        }
        for (int i = 0; i < 2 && e == cudaSuccess; ++i)
            e = cudaMalloc(&a->scratch64[i], sizeof(double) * kRec64 * np);
    }
    return e;
}

void drop_backward_graph(mpm_adjoint* a) {
    if (a->bgraph) cudaGraphExecDestroy(a->bgraph);
    a->bgraph = nullptr;
    a->bg_T = -1;
}

void free_observations(mpm_adjoint* a) {
    for (float4* p : a->obs) cudaFree(p);
    a->obs.clear();
    a->obs_steps.clear();
    a->obs_seeded = false;
}

void free_adjoint(mpm_adjoint* a) {
    drop_backward_graph(a);
    free_observations(a);
    cudaFree(a->obs_scale);
    cudaFree(a->obs_loss);
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
// memsets, device copies and event dependencies only, so it can be
// captured): for each checkpoint segment from the last, recompute its states
// and updated grids (unless the forward or a full tape kept them), then run
// its adjoint substeps in reverse, adding the seeds at their substeps.
// With two tape sets and a second stream `rs` (ev: 5 events), the recompute
// runs on `rs` one segment ahead: segment j - 1 is recomputed into one set
// while the adjoint of segment j reads the other; the recompute of j - 1
// waits for the adjoint of j + 1 (the last reader of its set), the adjoint of
// j for the recompute of j.  rs == st (or one set) runs them in turn.
// *cur_out: the adjoint buffer that ends up holding dL/dS_0.
int enqueue_backward(mpm_adjoint* a, const int* seed_steps, int nseeds, cudaStream_t st,
                     cudaStream_t rs, cudaEvent_t* ev, int* cur_out) {
    mpm_batch* b = a->b;
    const int n = b->n, S = (int)b->consts.size();
    const bool f64 = a->tape == MPM_TAPE_FP64;
    const bool overlap = rs != nullptr && rs != st && a->sets == 2;
    cudaStream_t r = overlap ? rs : st;
    cudaEvent_t* ev_rec = overlap ? ev : nullptr;      // [set]: recompute into it done
    cudaEvent_t* ev_adj = overlap ? ev + 2 : nullptr;  // [set]: adjoint of its segment done
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
    auto seg_range = [&](int j, int& t0, int& t1) {
        t0 = j * a->every;
        t1 = t0 + a->every < a->T ? t0 + a->every : a->T;
    };
    auto recomputed = [&](int j) { return !full_tape(a) && !(a->last_taped && j == nseg - 1); };
    // recompute segment j on stream r into its tape set: states and updated
    // grids of every substep
    auto recompute = [&](int j) -> int {
        if (!recomputed(j)) return MPM_OK;
        const int k = tape_set(a, j);
        if (overlap && j + 2 <= nseg - 1) MPM_CUDA(cudaStreamWaitEvent(r, ev_adj[k], 0));
        int t0 = 0, t1 = 0;
        seg_range(j, t0, t1);
        if (f64) {
            const double* curS = a->ckpt64[(size_t)j];
            for (int t = t0; t < t1; ++t) {
                double* dst = t + 1 < t1 ? a->seg64[k][(size_t)(t + 1 - t0)] : a->scratch64[0];
                launch_substep64(curS, a->gtape64[k] + (size_t)(t - t0) * nc, dst, a->scenes_d, S,
                                 a->pscene_d, n, a->ncells, r);
                curS = dst;
            }
        } else {
            if (cudaError_t e = batch_load_device(b, a->ckpt[(size_t)j], r); e != cudaSuccess)
                return cuda_fail(e, "mpm_backward recompute");
            for (int t = t0; t < t1; ++t) {
                if (sorted_step(b->sorted, &b->ps, b->posvel, b->counters, b->consts[0], 1, r,
                                &b->prof, b->graph) != 0)
                    return fail(MPM_E_CUDA, std::string("backward recompute: ") + sorted_error());
                b->stepped = true;
                // the updated grid, and the state after the substep when the
                // segment goes on, in one launch
                int4* gt = a->gtape[k] + (size_t)(t - t0) * nc;
                const int rc = t + 1 < t1
                                   ? sorted_export_all_canonical(b->sorted, gt, b->ps,
                                                                 a->seg[k][(size_t)(t + 1 - t0)],
                                                                 n, r, &b->prof)
                                   : sorted_export_all(b->sorted, gt, r, &b->prof);
                if (rc != 0)
                    return fail(MPM_E_CUDA, std::string("backward recompute: ") + sorted_error());
            }
        }
        if (overlap) MPM_CUDA(cudaEventRecord(ev_rec[k], r));
        return MPM_OK;
    };
    // the adjoint substeps of segment j in reverse, on st
    auto adjoint = [&](int j) -> int {
        const int k = tape_set(a, j);
        if (overlap && recomputed(j)) MPM_CUDA(cudaStreamWaitEvent(st, ev_rec[k], 0));
        int t0 = 0, t1 = 0;
        seg_range(j, t0, t1);
        const size_t g0 = full_tape(a) ? (size_t)t0 : 0;  // tape grid of substep t0
        for (int t = t1 - 1; t >= t0; --t) {
            if (f64) {
                const double* Sx = t == t0 ? a->ckpt64[(size_t)j] : a->seg64[k][(size_t)(t - t0)];
                launch_adjoint_substep64(Sx, a->gtape64[k] + (g0 + (size_t)(t - t0)) * nc,
                                         a->adj[cur], a->adj[cur ^ 1], a->gadj, a->scenes_d, S,
                                         a->pscene_d, n, a->ncells, a->pgrad_d, a->sort, st);
            } else {
                const Particles& Sx = t == t0 ? a->ckpt[(size_t)j] : a->seg[k][(size_t)(t - t0)];
                launch_adjoint_substep(Sx, a->gtape[k] + (g0 + (size_t)(t - t0)) * nc, a->adj[cur],
                                       a->adj[cur ^ 1], a->gadj, a->scenes_d, S, a->pscene_d, n,
                                       a->ncells, a->pgrad_d, a->sort, st);
            }
            cur ^= 1;
            add_seeds(t, a->adj[cur]);
        }
        if (overlap) MPM_CUDA(cudaEventRecord(ev_adj[k], st));
        return MPM_OK;
    };
    int rc = MPM_OK;
    if (overlap) {  // fork the recompute stream off st
        MPM_CUDA(cudaEventRecord(ev[4], st));
        MPM_CUDA(cudaStreamWaitEvent(r, ev[4], 0));
        if (nseg > 0) rc = recompute(nseg - 1);
        for (int j = nseg - 1; j >= 0 && rc == MPM_OK; --j) {
            if (j > 0) rc = recompute(j - 1);
            if (rc == MPM_OK) rc = adjoint(j);
        }
        // join it back, also after a failure (a capture must end joined)
        const cudaError_t e1 = cudaEventRecord(ev[4], r);
        const cudaError_t e2 = cudaStreamWaitEvent(st, ev[4], 0);
        if (rc != MPM_OK) return rc;
        MPM_CUDA(e1);
        MPM_CUDA(e2);
    } else {
        for (int j = nseg - 1; j >= 0 && rc == MPM_OK; --j) {
            rc = recompute(j);
            if (rc == MPM_OK) rc = adjoint(j);
        }
        if (rc != MPM_OK) return rc;
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

// At least `count` seed buffers (device streams kept between calls: a
// captured backward reads them at fixed addresses).
int ensure_seed_buffers(mpm_adjoint* a, int count) {
    while ((int)a->seedbuf.size() < count) {
        drop_backward_graph(a);
        Particles P{};
        const cudaError_t e = alloc_particles(P, (size_t)(a->b->n > 0 ? a->b->n : 1));
        if (e != cudaSuccess) {
            free_particles(P);
            return cuda_fail(e, "mpm_backward seeds");
        }
        a->seedbuf.push_back(P);
    }
    return MPM_OK;
}

// The backward of the last forward with seedbuf[i] added at substep
// steps[i]: replays the captured graph when (T, interval, tape, seed
// substeps) match the last capture, else captures it (plain launches while
// kernels are profiled); then reads the gradients back.  Synchronizes.
int run_backward(mpm_adjoint* a, const std::vector<int>& steps, float* grad_init,
                 double* grad_params, cudaStream_t st) {
    mpm_batch* b = a->b;
    const int n = b->n, S = (int)b->consts.size(), nseeds = (int)steps.size();
    int cur = 0;
    if (b->prof.enabled) {  // per-launch profiling: no graph, one stream
        if (int rc = enqueue_backward(a, steps.data(), nseeds, st, st, nullptr, &cur)) return rc;
    } else if (a->bgraph && a->bg_T == a->T && a->bg_every == a->every && a->bg_tape == a->tape &&
               a->bg_last_taped == a->last_taped && a->bg_steps == steps) {
        MPM_CUDA(cudaGraphLaunch(a->bgraph, st));
        cur = a->bg_cur;
    } else {
        drop_backward_graph(a);
        // capture stream, recompute stream and the events that order them
        cudaStream_t cs = nullptr, rs = nullptr;
        cudaEvent_t ev[5] = {};
        cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&rs, cudaStreamNonBlocking);
        for (int i = 0; i < 5 && e == cudaSuccess; ++i)
            e = cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming);
        const bool engine_graph = b->graph;
        b->graph = false;  // the engine's kernels go straight into this graph
        cudaGraph_t graph = nullptr;
        int rc = 0;
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            rc = enqueue_backward(a, steps.data(), nseeds, cs, rs, ev, &cur);
            e = cudaStreamEndCapture(cs, &graph);
        }
        b->graph = engine_graph;
        cudaGraphExec_t exec = nullptr;
        if (e == cudaSuccess && rc == 0) e = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        for (cudaEvent_t x : ev)
            if (x) cudaEventDestroy(x);
        if (rs) cudaStreamDestroy(rs);
        if (cs) cudaStreamDestroy(cs);
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
    a->obs_seeded = false;
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
            double4* G = a->gtape64[0] + (full_tape(a) ? (size_t)t * nc : 0);
            if (tape_last && t >= last_t0) {
                G = a->gtape64[0] + (size_t)(t - last_t0) * nc;
                if (t + 1 < substeps) dst = a->seg64[0][(size_t)(t + 1 - last_t0)];
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
                int4* gt = a->gtape[0] + (size_t)(t - last_t0) * nc;
                ++t;
                const Particles& dst = t < substeps ? a->seg[0][(size_t)(t - last_t0)]
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
                if (sorted_export_all_canonical(b->sorted, a->gtape[0] + (size_t)t * (size_t)a->ncells,
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
    MPM_CUDA(cudaStreamSynchronize(st));
    if (int rc = ensure_seed_buffers(a, nseeds)) return rc;
    a->obs_seeded = false;  // the buffers now hold these seeds
    for (int i = 0; i < nseeds; ++i)
        MPM_CUDA(upload_records(a->seedbuf[(size_t)i], seeds[i], b->n, a->stage, st));
    return run_backward(a, std::vector<int>(seed_steps, seed_steps + nseeds), grad_init,
                        grad_params, st);
}

int mpm_adjoint_set_observations(mpm_adjoint* a, int count, const int* substeps,
                                 const float* const* obs_xyz) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (count < 0 || (count > 0 && (!substeps || !obs_xyz)))
        return fail(MPM_E_INVALID, "bad observations");
    const int n = a->b->n;
    for (int i = 0; i < count; ++i) {
        if (!obs_xyz[i] && n) return fail(MPM_E_INVALID, "null observation block");
        if (substeps[i] < 0 || substeps[i] > a->max_substeps)
            return fail(MPM_E_INVALID, "observed substep outside [0, max_substeps]");
    }
    DeviceGuard g(a->b->device);
    MPM_CUDA(cudaDeviceSynchronize());
    free_observations(a);
    const size_t np = (size_t)(n > 0 ? n : 1);
    std::vector<float4> h(np);
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < count && e == cudaSuccess; ++i) {
        float4* d = nullptr;
        e = cudaMalloc(&d, sizeof(float4) * np);
        if (e != cudaSuccess) break;
        a->obs.push_back(d);
        a->obs_steps.push_back(substeps[i]);
        for (int j = 0; j < n; ++j)
            h[(size_t)j] = make_float4(obs_xyz[i][3 * (size_t)j], obs_xyz[i][3 * (size_t)j + 1],
                                       obs_xyz[i][3 * (size_t)j + 2], 0.0f);
        e = cudaMemcpy(d, h.data(), sizeof(float4) * (size_t)n, cudaMemcpyHostToDevice);
    }
    const int S = (int)a->b->consts.size();
    if (e == cudaSuccess && !a->obs_scale) e = cudaMalloc(&a->obs_scale, sizeof(float) * (size_t)S);
    if (e == cudaSuccess && !a->obs_loss) e = cudaMalloc(&a->obs_loss, sizeof(double) * (size_t)S);
    if (e != cudaSuccess) {  // no partial set of observations
        free_observations(a);
        return cuda_fail(e, "mpm_adjoint_set_observations");
    }
    std::vector<float> scale((size_t)S);
    for (int s = 0; s < S; ++s) {
        const int ns = a->b->desc[(size_t)s].num_particles;
        scale[(size_t)s] = ns > 0 ? (float)(2.0 / ns) : 0.0f;
    }
    MPM_CUDA(cudaMemcpy(a->obs_scale, scale.data(), sizeof(float) * (size_t)S,
                        cudaMemcpyHostToDevice));
    return MPM_OK;
}

int mpm_adjoint_observation_loss(mpm_adjoint* a, double* loss_per_scene, void* stream) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (a->T < 0) return fail(MPM_E_STATE, "no forward run");
    mpm_batch* b = a->b;
    const int n = b->n, S = (int)b->consts.size(), count = (int)a->obs.size();
    for (int i = 0; i < count; ++i)
        if (ckpt_slot(a, a->obs_steps[(size_t)i], a->T) < 0)
            return fail(MPM_E_INVALID, "an observed substep is not a checkpoint of the last forward");
    DeviceGuard g(b->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MPM_CUDA(cudaStreamSynchronize(st));
    if (int rc = ensure_seed_buffers(a, count)) return rc;
    if (S > 0) MPM_CUDA(cudaMemsetAsync(a->obs_loss, 0, sizeof(double) * (size_t)S, st));
    for (int i = 0; i < count; ++i) {
        const int j = ckpt_slot(a, a->obs_steps[(size_t)i], a->T);
        const bool f64 = a->tape == MPM_TAPE_FP64;
        launch_obs_loss(f64 ? nullptr : &a->ckpt[(size_t)j], f64 ? a->ckpt64[(size_t)j] : nullptr,
                        a->obs[(size_t)i], a->pscene_d, a->obs_scale, a->seedbuf[(size_t)i],
                        a->obs_loss, n, st);
    }
    MPM_CUDA(cudaGetLastError());
    std::vector<double> sums((size_t)S, 0.0);
    if (S > 0)
        MPM_CUDA(cudaMemcpyAsync(sums.data(), a->obs_loss, sizeof(double) * (size_t)S,
                                 cudaMemcpyDeviceToHost, st));
    MPM_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < S && loss_per_scene; ++s) {
        const int ns = b->desc[(size_t)s].num_particles;
        loss_per_scene[s] = ns > 0 ? sums[(size_t)s] / ns : 0.0;
    }
    a->obs_seeded = true;
    return MPM_OK;
}

int mpm_backward_observed(mpm_adjoint* a, float* grad_init, double* grad_params, void* stream) {
    if (!a) return fail(MPM_E_INVALID, "null adjoint handle");
    if (a->T < 0) return fail(MPM_E_STATE, "no forward run");
    if (!a->obs_seeded)
        return fail(MPM_E_STATE, "no observation loss since the last forward");
    DeviceGuard g(a->b->device);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    MPM_CUDA(cudaStreamSynchronize(st));
    return run_backward(a, a->obs_steps, grad_init, grad_params, st);
}

}  // extern "C"
