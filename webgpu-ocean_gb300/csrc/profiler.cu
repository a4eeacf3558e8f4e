// profiler.cu -- launch accounting for both engines (LaunchProfiler).
#include <cstdlib>

#include "mpm_internal.h"

namespace mpm {

const char* kernel_name(int id) {
    static const char* names[KID_COUNT] = {
        "clearGrid", "p2g_1", "p2g_2", "updateGrid", "g2p", "copyPosition",
        "bin", "scan", "scatter", "sorted_p2g_1", "sorted_p2g_2", "sorted_g2p_p2g_1",
        "export_grid", "canonicalize"};
    return (id >= 0 && id < KID_COUNT) ? names[id] : "?";
}

namespace {
cudaEvent_t take(LaunchProfiler& p) {
    if (p.npool > 0) return p.pool[--p.npool];
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}
void give(LaunchProfiler& p, cudaEvent_t e) {
    if (!e) return;
    if (p.npool == p.pool_cap) {
        const int nc = p.pool_cap ? 2 * p.pool_cap : 64;
        void* q = std::realloc(p.pool, sizeof(cudaEvent_t) * nc);
        if (!q) { cudaEventDestroy(e); return; }
        p.pool = static_cast<cudaEvent_t*>(q);
        p.pool_cap = nc;
    }
    p.pool[p.npool++] = e;
}
}  // namespace

void LaunchProfiler::before(cudaStream_t st) {
    if (!enabled) return;
    open = take(*this);
    if (open) cudaEventRecord(open, st);
}

void LaunchProfiler::after(int id, cudaStream_t st) {
    ++launches[id];
    if (!enabled || !open) return;
    cudaEvent_t b = take(*this);
    if (!b) { give(*this, open); open = nullptr; return; }
    cudaEventRecord(b, st);
    if (npending == cap) {
        const int nc = cap ? 2 * cap : 256;
        void* q = std::realloc(pending, sizeof(Pending) * nc);
        if (!q) { give(*this, open); give(*this, b); open = nullptr; return; }
        pending = static_cast<Pending*>(q);
        cap = nc;
    }
    pending[npending++] = Pending{id, open, b};
    open = nullptr;
}

int LaunchProfiler::collect() {
    int rc = 0;
    for (int i = 0; i < npending; ++i) {
        Pending& q = pending[i];
        float ms = 0.f;
        if (cudaEventSynchronize(q.b) == cudaSuccess && cudaEventElapsedTime(&ms, q.a, q.b) == cudaSuccess) {
            total_ms[q.id] += ms;
            ++timed[q.id];
        } else {
            rc = -1;
        }
        give(*this, q.a);
        give(*this, q.b);
    }
    npending = 0;
    return rc;
}

void LaunchProfiler::reset() {
    collect();
    for (int i = 0; i < KID_COUNT; ++i) launches[i] = 0, total_ms[i] = 0.0, timed[i] = 0;
}

void LaunchProfiler::release() {
    collect();
    for (int i = 0; i < npool; ++i) cudaEventDestroy(pool[i]);
    std::free(pool);
    std::free(pending);
    pool = nullptr;
    pending = nullptr;
    npool = pool_cap = npending = cap = 0;
}

}  // namespace mpm
