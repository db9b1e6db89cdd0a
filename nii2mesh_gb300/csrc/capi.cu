// capi.cu — host orchestration of the meshify pipeline and the C ABI.
//
// meshify (src/meshify.c:286-389) on the GPU, stage by stage:
//   1. pre-smooth fused with range + bbox (smooth.cu), or a range/bbox pass
//   2. one readback: range, isolevel fallback, non-finite check
//   3. optional clustering (label.cu), range/bbox recomputed afterwards
//   4. marching cubes count pass + scan (mc.cu / oldcubes.cu), readback of
//      the vertex/triangle totals, emit pass straight into vec3d/vec3i
//   5. weld: the few near-grid-point candidates are read back and grouped on
//      the host with the reference's greedy rule; merges applied on device
//   6. degenerate-triangle removal and compaction (mesh.cu)
// Edge darkening is applied on the fly by the marching-cubes value fetch.
#include <stdarg.h>
#include <stdint.h>
#include <sys/mman.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <ctime>
#include <condition_variable>
#include <mutex>
#include <thread>
#include <unordered_set>
#include <vector>

#include "n2m_internal.cuh"

// ---- errors, counters -------------------------------------------------------------
static thread_local char g_err[512] = "";
std::atomic<long long> g_n2m_launches{0};

extern "C" long long n2m_kernel_launches(void) { return g_n2m_launches.load(); }

void n2m_set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

extern "C" const char *n2m_last_error(void) { return g_err; }

extern "C" const char *n2m_status_string(int s) {
    static const char *names[] = {"ok",         "no CUDA device",   "CUDA error",      "out of memory",
                                  "bad arguments", "no variability", "empty mesh",      "non-finite voxels",
                                  "too large",  "device wait timed out", "internal error"};
    return (s >= 0 && s <= 10) ? names[s] : "unknown";
}

// host-side fault injection (tests): the k-th device allocation from now fails, once
static std::atomic<int> g_fail_alloc{-1};
extern "C" int n2m_debug_fail_allocations(int after) { return g_fail_alloc.exchange(after < 0 ? -1 : after); }

n2m_status DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return N2M_OK;
    int k = g_fail_alloc.load();
    while (k >= 0 && !g_fail_alloc.compare_exchange_weak(k, k - 1)) {
    }
    if (k == 0) {
        release();
        n2m_set_error("allocation of %zu bytes failed (injected)", bytes);
        return N2M_ERR_OOM;
    }
    release();
    size_t want = bytes + bytes / 8 + 256;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        cap = 0;
        n2m_set_error("cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
        return N2M_ERR_OOM;
    }
    cap = want;
    return N2M_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

// ---- context ------------------------------------------------------------------------
// Output buffers of a host-memory meshify call.  They are malloc'd (the
// caller frees them with free(), as the reference's callers do) before the
// GPU work starts (sized like the last call's mesh) or as soon as the raw
// mesh size is known, and their pages are faulted in by a pool of host
// threads while the GPU works: first-touch page faults of a fresh 100+ MB
// buffer cost more than the device-to-host copy itself.
// ask for transparent huge pages on the 2 MB-aligned interior of a buffer
// (512x fewer page faults where the kernel allows it; a no-op otherwise)
inline void advise_huge(void *p, size_t n) {
    const uintptr_t a = ((uintptr_t)p + (2u << 20) - 1) & ~(uintptr_t)((2u << 20) - 1), e = ((uintptr_t)p + n) & ~(uintptr_t)((2u << 20) - 1);
    if (e > a) madvise((void *)a, e - a, MADV_HUGEPAGE);
}

struct HostOut {
    char *pts = nullptr, *tris = nullptr;
    size_t pb = 0, tb = 0;
    // worker pool, created on first use and kept for the context's lifetime
    std::vector<std::thread> pool;
    std::mutex mu;
    std::condition_variable cv_job, cv_done;
    unsigned long long job = 0;   // generation of the current job
    int pending = 0;              // workers still busy with it
    bool quit = false;
    void work(int i, int n) {
        unsigned long long seen = 0;
        for (;;) {
            char *p, *t;
            size_t a, b;
            {
                std::unique_lock<std::mutex> lk(mu);
                cv_job.wait(lk, [&] { return quit || job != seen; });
                if (quit) return;
                seen = job;
                p = pts;
                t = tris;
                a = pb;
                b = tb;
            }
            const size_t page = 4096, total = a + b, lo = total * i / n, hi = total * (i + 1) / n;
            for (size_t o = (lo + page - 1) / page * page; o < hi; o += page) {
                if (o < a) p[o] = 0;
                else t[o - a] = 0;
            }
            std::lock_guard<std::mutex> lk(mu);
            if (--pending == 0) cv_done.notify_all();
        }
    }
    void start(size_t pbytes, size_t tbytes) {
        discard();
        pts = (char *)malloc(pbytes);
        tris = (char *)malloc(tbytes);
        if (!pts || !tris) {
            free(pts);
            free(tris);
            pts = tris = nullptr;
            return;
        }
        pb = pbytes;
        tb = tbytes;
        advise_huge(pts, pb);
        advise_huge(tris, tb);
        if (pool.empty()) {
            const unsigned hw = std::thread::hardware_concurrency();   // leave two cores to the calling thread
            const int n = (int)std::min(16u, std::max(1u, hw > 2 ? hw - 2 : 1u));
            try {
                for (int i = 0; i < n; i++) pool.emplace_back([this, i, n] { work(i, n); });
            } catch (...) {   // fewer workers (or none: the copy then faults the pages in itself)
            }
        }
        if (pool.empty()) return;
        std::lock_guard<std::mutex> lk(mu);
        pending = (int)pool.size();
        job++;
        cv_job.notify_all();
    }
    void join() {
        std::unique_lock<std::mutex> lk(mu);
        cv_done.wait(lk, [&] { return pending == 0; });
    }
    void discard() {
        join();
        free(pts);
        free(tris);
        pts = tris = nullptr;
        pb = tb = 0;
    }
    ~HostOut() {
        discard();
        {
            std::lock_guard<std::mutex> lk(mu);
            quit = true;
        }
        cv_job.notify_all();
        for (auto &t : pool) t.join();
    }
};

struct n2m_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t evs[8] = {};   // stage boundaries of the last pipeline run
    cudaEvent_t eva[2] = {};   // around pass A of the exact-on-demand pre-smooth
    bool pass_a = false;       // whether the last pipeline run used it
    DevBuf in, raw, vol, stmp, stmp2, stats, totals, cand, ncand, ocq, lubits, pts_raw, tris_raw, pts, tris, ntf, weld,
        gath, hmesh;
    OdWork od;   // pre-smooth with exact rounding on demand
    McWork mc;
    ScanWork scan;
    LabelWork lab;
    LabelPost lpost{};
    DegWork deg;
    HcWork hc;
    ThresholdWork th;
    void *pinned = nullptr;   // small readbacks
    DevBuf gA, gB, gs, gtmp;   // adjoint scratch
    AtlasWork aw;
    DevBuf alab, lpts, ltris;   // atlas input copy, per-label-loop output
    std::vector<n2m_atlas_mesh> atlas_meshes;
    // state of the last forward run that the adjoint needs
    struct {
        bool valid = false, smoothed = false, clustered = false;
        int cubes = 0, nv_raw = 0, post_smooth = 0, nrem = 0, nov = 0;
        int dim[3] = {0, 0, 0};
        McGrid g;
        McCounts mcn;
        const int *removed = nullptr, *ov_id = nullptr, *ov_src = nullptr;
    } fwd;
    // result of the last pipeline run (device pointers into the buffers above)
    vec3d *res_pts = nullptr;
    vec3i *res_tris = nullptr;
    int res_np = 0, res_nt = 0;
    // host-memory calls: staged input upload and pre-faulted outputs
    cudaStream_t copy = nullptr;
    StagedInput stage;
    bool want_host = false;
    HostOut hout;
    size_t hint_pb = 0, hint_tb = 0;   // raw mesh bytes of the last host-memory call (early pre-faulting)
    bool pts_early = false;            // the final vertices are already on their way to the host
    // n2m_meshify_into: caller-owned host output buffers (no allocation, no page faulting)
    vec3i *user_t = nullptr;
    vec3d *user_p = nullptr;
    size_t user_tcap = 0, user_pcap = 0;
    WriterWork wr;                     // mesh writers
};

extern "C" int n2m_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

extern "C" n2m_status n2m_context_create(n2m_context **out, int device) {
    if (!out) return N2M_ERR_BAD_ARGS;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || device < 0 || device >= n) {
        cudaGetLastError();
        n2m_set_error("no usable CUDA device (count %d, requested %d)", n, device);
        return N2M_ERR_NO_DEVICE;
    }
    n2m_context *c = new n2m_context;
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        cudaMallocHost(&c->pinned, 4096) != cudaSuccess) {
        n2m_set_error("context creation failed: %s", cudaGetErrorString(cudaGetLastError()));
        delete c;
        return N2M_ERR_CUDA;
    }
    for (int i = 0; i < 8; i++)
        if (cudaEventCreate(&c->evs[i]) != cudaSuccess || (i < 2 && cudaEventCreate(&c->eva[i]) != cudaSuccess)) {
            n2m_set_error("event creation failed");
            return N2M_ERR_CUDA;
        }
    if (cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking) != cudaSuccess) {
        n2m_set_error("stream creation failed");
        return N2M_ERR_CUDA;
    }
    c->stage.copy = c->copy;
    for (int i = 0; i <= N2M_STAGE_SLABS; i++)
        if (cudaEventCreateWithFlags(&c->stage.ev[i], cudaEventDisableTiming) != cudaSuccess) {
            n2m_set_error("event creation failed");
            return N2M_ERR_CUDA;
        }
    *out = c;
    return N2M_OK;
}

extern "C" void n2m_context_destroy(n2m_context *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    DevBuf *bufs[] = {&c->aw.cnt, &c->aw.bb, &c->aw.boxes, &c->aw.queue, &c->aw.arena, &c->aw.mask, &c->aw.keep,
                      &c->aw.lab, &c->aw.edge, &c->aw.ucnt, &c->aw.words, &c->aw.counts, &c->aw.active, &c->aw.tot,
                      &c->aw.pts, &c->aw.pts2, &c->aw.tris, &c->aw.tris2, &c->aw.cand, &c->aw.gath, &c->aw.weld,
                      &c->aw.ranges, &c->alab, &c->lpts, &c->ltris, &c->gA, &c->gB, &c->gs, &c->gtmp, &c->in, &c->raw, &c->vol, &c->stmp, &c->stats, &c->totals, &c->cand, &c->ncand, &c->ocq, &c->pts_raw,
                      &c->tris_raw, &c->pts, &c->tris, &c->ntf, &c->weld, &c->gath, &c->hmesh,
                      &c->mc.words, &c->mc.counts, &c->mc.cand, &c->mc.verts_tmp, &c->mc.tris_tmp, &c->mc.signs, &c->mc.ctr, &c->scan.part,
                      &c->lab.lab, &c->lab.mask, &c->lab.keep, &c->lab.cnt, &c->lab.edge, &c->lab.rc, &c->lab.misc,
                      &c->deg.flags, &c->deg.tmp, &c->hc.start, &c->hc.refs, &c->hc.fill, &c->hc.P, &c->hc.Q,
                      &c->hc.B, &c->hc.Lo, &c->hc.border, &c->hc.hasnb, &c->hc.bad, &c->th.buf, &c->th.table,
                      &c->stmp2, &c->lubits, &c->od.st, &c->od.unc, &c->od.cmin, &c->od.cmax, &c->od.need_z, &c->od.need_y,
                      &c->od.need_x, &c->od.off, &c->od.list, &c->od.lcnt, &c->od.vsign,
                      &c->wr.mt, &c->wr.mp, &c->wr.pack, &c->wr.pack2, &c->wr.lens, &c->wr.flag, &c->wr.out};
    for (DevBuf *b : bufs) b->release();
    deflate_release(c->wr.df);
    if (c->aw.exec) cudaGraphExecDestroy((cudaGraphExec_t)c->aw.exec);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->wr.host) cudaFreeHost(c->wr.host);
    for (int i = 0; i < 8; i++)
        if (c->evs[i]) cudaEventDestroy(c->evs[i]);
    for (int i = 0; i < 2; i++)
        if (c->eva[i]) cudaEventDestroy(c->eva[i]);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    c->hout.discard();
    if (c->copy) {
        cudaStreamSynchronize(c->copy);
        cudaStreamDestroy(c->copy);
    }
    for (int i = 0; i <= N2M_STAGE_SLABS; i++)
        if (c->stage.ev[i]) cudaEventDestroy(c->stage.ev[i]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" void *n2m_context_stream(n2m_context *c) { return c ? (void *)c->stream : nullptr; }

namespace {
// per-thread default context for the drop-in entry points
struct TlsCtx {
    n2m_context *c = nullptr;
    ~TlsCtx() { n2m_context_destroy(c); }
};
thread_local TlsCtx g_tls;
int g_oldcubes = 0;
thread_local bool g_quiet = false;   // atlas runs do not print per-label messages

n2m_status default_ctx(n2m_context **c) {
    if (!g_tls.c) {
        const char *d = getenv("N2M_DEVICE");
        CKS(n2m_context_create(&g_tls.c, d ? atoi(d) : 0));
    }
    *c = g_tls.c;
    return N2M_OK;
}

template <class T> n2m_status readback(n2m_context *c, T *dst, const void *dsrc, size_t n = 1) {
    CK(cudaMemcpyAsync(c->pinned, dsrc, n * sizeof(T), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    memcpy(dst, c->pinned, n * sizeof(T));
    return N2M_OK;
}

__global__ void k_gather(const vec3d *__restrict__ p, const int *__restrict__ ids, int n, vec3d *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = p[ids[i]];
}

// corner q = 3*t + c of the triangle list takes vertex v, for n (q, v) pairs
__global__ void k_set_corners(vec3i *tris, const int2 *__restrict__ qv, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const int t = qv[i].x / 3, c = qv[i].x - 3 * t;
        int *T = &tris[t].x;
        T[c] = qv[i].y;
    }
}

double dist3(const vec3d &a, const vec3d &b) {
    const double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
    return sqrt(dx * dx + dy * dy + dz * dz);
}

uint32_t key_bits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

struct Prep {
    const float *vol;
    float iso, mn, mnp, edge_max;
    int lo[3], hi[3];
    bool od = false;          // vol is smoothed approximately: marching cubes makes it exact where it reads it
    const float *src = nullptr;
    const LabelPost *post = nullptr;   // with od: what the clustering did to vol
};

// The reference's greedy grouping (src/meshify.c:62-78) over elements with
// positions pos and reference order `order`: sorted by (float distance to v0,
// order) as its stable radix sort leaves them, each element not yet in a group
// seeds a new one that takes every later element within the tolerance, even
// one already in an earlier group.  Returns the group of every element.
std::vector<int> weld_groups(const std::vector<vec3d> &pos, const std::vector<long long> &order, vec3d v0, int *ng_out) {
    const int n = (int)pos.size();
    std::vector<float> key(n);
    std::vector<int> srt(n);
    for (int i = 0; i < n; i++) {
        key[i] = (float)dist3(v0, pos[i]);
        srt[i] = i;
    }
    std::sort(srt.begin(), srt.end(), [&](int a, int b) {
        const uint32_t ka = key_bits(key[a]), kb = key_bits(key[b]);
        return ka != kb ? ka < kb : order[a] < order[b];
    });
    const float tol = 0.00001f;
    std::vector<int> grp(n, -1);
    int ng = 0;
    for (int i = 0; i < n; i++) {
        const int a = srt[i];
        if (grp[a] >= 0) continue;
        for (int j = i; j < n && (key[srt[j]] - key[a]) < tol; j++)
            if (dist3(pos[a], pos[srt[j]]) < tol) grp[srt[j]] = ng;
        ng++;
    }
    *ng_out = ng;
    return grp;
}

// removed ids (with the id each merges into) and position overrides, sorted by id
void sort_weld_lists(std::vector<int> &removed, std::vector<int> &keep, std::vector<int> &ov_id,
                     std::vector<vec3d> &ov_pos, std::vector<int> &ov_src) {
    std::vector<int> ri(removed.size());
    for (size_t i = 0; i < ri.size(); i++) ri[i] = (int)i;
    std::sort(ri.begin(), ri.end(), [&](int a, int b) { return removed[a] < removed[b]; });
    std::vector<int> r2, k2;
    for (int i : ri) { r2.push_back(removed[i]); k2.push_back(keep[i]); }
    removed.swap(r2);
    keep.swap(k2);
    std::vector<int> oi(ov_id.size());
    for (size_t i = 0; i < oi.size(); i++) oi[i] = (int)i;
    std::sort(oi.begin(), oi.end(), [&](int a, int b) { return ov_id[a] < ov_id[b]; });
    std::vector<int> o2, s2;
    std::vector<vec3d> p2;
    for (int i : oi) { o2.push_back(ov_id[i]); p2.push_back(ov_pos[i]); s2.push_back(ov_src[i]); }
    ov_id.swap(o2);
    ov_pos.swap(p2);
    ov_src.swap(s2);
}

// Host side of the weld (src/meshify.c:45-106) restricted to the candidates:
// only vertices within the tolerance of another vertex can merge, and every
// such vertex is a candidate, so the greedy grouping over the candidates makes
// exactly the reference's merges.  Lewiner's vertices are shared already, so
// each is one element in the reference's vertex order.  Outputs the removed
// ids (sorted), the id each merges into, and position overrides (the group's
// last writer in the reference's vertex order).
n2m_status weld_candidates(n2m_context *c, int nv, int ncand, std::vector<int> &removed, std::vector<int> &keep,
                           std::vector<int> &ov_id, std::vector<vec3d> &ov_pos, std::vector<int> &ov_src, vec3d v0) {
    std::vector<int> ids(ncand);
    CK(cudaMemcpyAsync(ids.data(), c->cand.p, ncand * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    std::sort(ids.begin(), ids.end());
    ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
    const int n = (int)ids.size();
    CKS(c->gath.ensure((size_t)n * (sizeof(vec3d) + sizeof(int))));
    vec3d *dpos = c->gath.as<vec3d>();
    int *dids = (int *)(dpos + n);
    CK(cudaMemcpyAsync(dids, ids.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    { k_gather<<<(n + 255) / 256, 256, 0, c->stream>>>(c->pts_raw.as<vec3d>(), dids, n, dpos); N2M_COUNT(); }
    CKL();
    std::vector<vec3d> pos(n);
    CK(cudaMemcpyAsync(pos.data(), dpos, n * sizeof(vec3d), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const std::vector<long long> order(ids.begin(), ids.end());   // the reference's vertex order
    int ng = 0;
    const std::vector<int> grp = weld_groups(pos, order, v0, &ng);
    // per group: keep the smallest id, position of the last writer
    std::vector<int> gkeep(ng, INT32_MAX), glast(ng, -1), gsize(ng, 0);
    for (int i = 0; i < n; i++) {
        const int g = grp[i];
        gsize[g]++;
        gkeep[g] = std::min(gkeep[g], ids[i]);
        if (glast[g] < 0 || order[i] > order[glast[g]]) glast[g] = i;
    }
    for (int i = 0; i < n; i++) {
        const int g = grp[i];
        if (gsize[g] < 2) continue;
        if (ids[i] != gkeep[g]) {
            removed.push_back(ids[i]);
            keep.push_back(gkeep[g]);
        } else if (glast[g] != i) {
            ov_id.push_back(ids[i]);
            ov_pos.push_back(pos[glast[g]]);
            ov_src.push_back(ids[glast[g]]);
        }
    }
    sort_weld_lists(removed, keep, ov_id, ov_pos, ov_src);
    (void)nv;
    return N2M_OK;
}

// The oldcubes weld.  The reference welds a triangle soup: every triangle
// corner is its own copy of a vertex, at the position the emitting cube's
// VertexInterp gives (the edge's orientation in that cube), with its own key
// and its order 3*t + c; the soup's first copy is the origin of the keys.  So
// the copies of the candidates are the elements here, and a vertex whose
// copies land in different groups is split: every candidate corner gets its
// group's vertex (corners: (3*t + c, vertex) pairs), the group's vertex is
// the smallest member not already another group's, at the position of the
// group's last copy; members that are no group's vertex are removed.
n2m_status weld_oc(n2m_context *c, const Prep &P, const int dim[3], int nv, int nt, int ncand, std::vector<int> &removed,
                   std::vector<int> &keep, std::vector<int> &ov_id, std::vector<vec3d> &ov_pos, std::vector<int> &ov_src,
                   std::vector<int2> &corners) {
    CKS(c->lubits.ensure(((size_t)nv + 31) / 32 * sizeof(unsigned)));
    unsigned cap = (unsigned)std::min<long long>(32LL * ncand + 1024, 3LL * nt), ncopy = 0;
    unsigned *dq = nullptr, *dcount = nullptr;
    for (int pass = 0; pass < 2; pass++) {   // a second pass with room for every copy the first one counted
        CKS(c->ocq.ensure(((size_t)cap + 2) * sizeof(unsigned)));
        dq = c->ocq.as<unsigned>();
        dcount = dq + cap + 1;
        CKS(oc_copies(c->tris_raw.as<vec3i>(), nt, nv, c->cand.as<int>(), ncand, c->lubits.as<unsigned>(), dq, dcount,
                      cap, c->stream));
        CKS(readback(c, &ncopy, dcount));
        if (ncopy <= cap) break;
        cap = ncopy;
    }
    if (ncopy > cap) {
        n2m_set_error("weld copy overflow (%u > %u)", ncopy, cap);
        return N2M_ERR_INTERNAL;
    }
    CK(cudaMemsetAsync(dq + ncopy, 0, sizeof(unsigned), c->stream));   // q = 0: the soup's first copy, the origin
    const int n = (int)ncopy + 1;
    CKS(c->gath.ensure((size_t)n * (sizeof(vec3d) + sizeof(int))));
    vec3d *dpos = c->gath.as<vec3d>();
    int *dvid = (int *)(dpos + n);
    CKS(oc_copy_positions(P.vol, dim, P.lo, P.hi, P.iso, P.edge_max, c->mc, c->tris_raw.as<vec3i>(), dq, n, dvid, dpos,
                          c->stream));
    std::vector<unsigned> q(n);
    std::vector<int> vid(n);
    std::vector<vec3d> pos(n);
    CK(cudaMemcpyAsync(q.data(), dq, n * sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(vid.data(), dvid, n * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(pos.data(), dpos, n * sizeof(vec3d), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    const vec3d v0 = pos[ncopy];
    q.pop_back();
    vid.pop_back();
    pos.pop_back();
    const std::vector<long long> order(q.begin(), q.end());
    int ng = 0;
    const std::vector<int> grp = weld_groups(pos, order, v0, &ng);
    std::vector<int> glast(ng, -1);
    std::vector<std::vector<int>> gv(ng);   // member vertices of each group
    for (int i = 0; i < (int)ncopy; i++) {
        const int g = grp[i];
        if (glast[g] < 0 || q[i] > q[glast[g]]) glast[g] = i;
        gv[g].push_back(vid[i]);
    }
    std::vector<int> rep(ng, -1);
    std::unordered_set<int> taken;
    for (int g = 0; g < ng; g++) {
        if (glast[g] < 0) continue;   // every member moved on to a later group
        std::sort(gv[g].begin(), gv[g].end());
        for (int v : gv[g])
            if (!taken.count(v)) {
                rep[g] = v;
                break;
            }
        if (rep[g] < 0) {
            n2m_set_error("weld: a group with no vertex of its own");
            return N2M_ERR_INTERNAL;
        }
        taken.insert(rep[g]);
        ov_id.push_back(rep[g]);
        ov_pos.push_back(pos[glast[g]]);
        ov_src.push_back(rep[g]);
    }
    std::unordered_set<int> seen;
    for (int i = 0; i < (int)ncopy; i++) {
        const int r = rep[grp[i]];
        if (vid[i] != r) corners.push_back(make_int2((int)q[i], r));
        if (!taken.count(vid[i]) && seen.insert(vid[i]).second) {
            removed.push_back(vid[i]);
            keep.push_back(r);
        }
    }
    sort_weld_lists(removed, keep, ov_id, ov_pos, ov_src);
    return N2M_OK;
}

float half_sum(float a, float b) {   // (float)(0.5 * (a + b)) with a float sum, as C evaluates it
    volatile float s = a + b;
    return (float)(0.5 * (double)s);
}


// stages 1-3: smoothing, range, clustering, bbox
n2m_status prepare(n2m_context *c, const float *d_src, const int dim[3], const n2m_options &o, bool verbose,
                   Prep &P, n2m_report *rep) {
    const int nx = dim[0], ny = dim[1], nz = dim[2];
    const size_t n = (size_t)nx * ny * nz;
    const bool smooth = o.pre_smooth && nx >= 5 && ny >= 5 && nz >= 5;
    const bool label = o.only_largest || o.fill_bubbles;
    float iso = o.isolevel;
    c->pass_a = false;
    CKS(c->stats.ensure(2 * sizeof(VolStats)));
    VolStats *dst = c->stats.as<VolStats>();
    VolStats h[2];
    stats_init_host(&h[0]);
    stats_init_host(&h[1]);
    CK(cudaMemcpyAsync(dst, h, 2 * sizeof(VolStats), cudaMemcpyHostToDevice, c->stream));
    float *vol = nullptr;
    if (smooth || label) {
        CKS(c->vol.ensure(n * sizeof(float)));
        vol = c->vol.as<float>();
    }
    if (!smooth && label) CK(cudaMemcpyAsync(vol, d_src, n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaEventRecord(c->evs[0], c->stream));
    // Volume already in device memory: exact rounding on demand (only where marching
    // cubes reads values), also under -l 1 clustering, whose mask is pass A's sign
    // bitmap and whose result's minimum is the volume's once any voxel is masked out.
    // Otherwise the exact three passes; a volume arriving from host memory in slabs is
    // smoothed while it arrives that way (the on-demand repair could only start after
    // the last slab)
    bool od = smooth && (!label || o.only_largest) && !c->stage.host && od_eligible(d_src, nx, ny, nz);
    if (smooth) {
        CKS(c->stmp.ensure(n * sizeof(float)));
        const StagedInput *stage = c->stage.host ? &c->stage : nullptr;
        if (od) {
            bool fallback = false;
            CK(cudaEventRecord(c->eva[0], c->stream));
            CKS(od_approx(d_src, vol, nx, ny, nz, iso, c->od, c->stream, stage));
            CK(cudaEventRecord(c->eva[1], c->stream));
            c->pass_a = true;
            CKS(od_resolve(d_src, vol, nx, ny, nz, iso, c->od, dst, c->stream, &fallback, label || o.cubes == N2M_CUBES_OLDCUBES));
            if (fallback) {   // the input is on the device by now
                od = false;
                CK(cudaMemcpyAsync(dst, h, sizeof(VolStats), cudaMemcpyHostToDevice, c->stream));
                CKS(launch_smooth(d_src, vol, c->stmp.as<float>(), nx, ny, nz, iso, dst, c->stream, nullptr));
            }
        } else {
            CKS(launch_smooth(d_src, vol, c->stmp.as<float>(), nx, ny, nz, iso, dst, c->stream, stage));
        }
    }
    else CKS(launch_stats(label ? vol : d_src, nx, ny, nz, iso, true, dst, c->stream));
    CK(cudaEventRecord(c->evs[1], c->stream));
    const float *v = vol ? vol : d_src;
    VolStats s0;
    CKS(readback(c, &s0, dst));
    if (s0.nonfinite) {
        n2m_set_error("%u non-finite voxels in the volume", s0.nonfinite);
        return N2M_ERR_NONFINITE;
    }
    const float mn = ord2f(s0.vmin), mx = ord2f(s0.vmax);
    if (mn == mx) {
        if (!g_quiet) printf("Error: No variability in image intensity.\n");
        n2m_set_error("no variability in image intensity");
        return N2M_ERR_NO_VARIABILITY;
    }
    bool stale = false;
    if (iso <= mn || iso > mx) {
        iso = half_sum(mn, mx);
        if (!g_quiet)
            printf("Suggested isolevel out of range. Intensity range %g..%g, setting isolevel to %g\n", mn, mx, iso);
        stale = true;
        if (od) {   // the approximate pass decided signs against the old isolevel: smooth exactly
            od = false;
            CKS(launch_smooth(d_src, vol, c->stmp.as<float>(), nx, ny, nz, iso, dst + 1, c->stream, nullptr));
        }
    }
    if (verbose) printf("intensity range %g..%g, isolevel %g\n", mn, mx, iso);
    VolStats s1 = s0;
    float min_after = mn;
    if (label) {
        // (a stale isolevel's exact smoothing above left its statistics there)
        CK(cudaMemcpyAsync(dst + 1, &h[1], sizeof(VolStats), cudaMemcpyHostToDevice, c->stream));
        CKS(run_labelling(vol, nx, ny, nz, iso, mn, o.only_largest, o.fill_bubbles, c->lab, dst + 1, c->stream,
                          od ? c->od.vsign.as<unsigned>() : nullptr, &c->lpost));
        CKS(readback(c, &s1, dst + 1));
        if (od && s1.masked == 0) {   // nothing masked out: the minimum is the labelled values': smooth exactly
            od = false;
            CK(cudaMemcpyAsync(dst, h, 2 * sizeof(VolStats), cudaMemcpyHostToDevice, c->stream));
            CKS(launch_smooth(d_src, vol, c->stmp.as<float>(), nx, ny, nz, iso, dst, c->stream, nullptr));
            CKS(run_labelling(vol, nx, ny, nz, iso, mn, o.only_largest, o.fill_bubbles, c->lab, dst + 1, c->stream));
            CKS(readback(c, &s1, dst + 1));
        }
        min_after = od ? mn : ord2f(s1.vmin);   // masked voxels hold mn, every exact value is >= mn
    } else if (stale) {
        CKS(launch_stats(v, nx, ny, nz, iso, false, dst + 1, c->stream));
        CKS(readback(c, &s1, dst + 1));
    }
    CK(cudaEventRecord(c->evs[2], c->stream));
    if (s1.lo[0] > s1.hi[0]) {
        n2m_set_error("no voxel at or above the isolevel");
        return N2M_ERR_EMPTY;
    }
    volatile float mi = mn + iso;
    P.edge_max = (float)(0.75 * (double)mi);
    P.mnp = fminf(min_after, P.edge_max);
    P.vol = v;
    P.iso = iso;
    P.mn = mn;
    P.od = od;
    P.src = d_src;
    P.post = od && label ? &c->lpost : nullptr;
    for (int i = 0; i < 3; i++) {
        P.lo[i] = std::max(s1.lo[i] - 1, 0);
        P.hi[i] = std::min(s1.hi[i] + 2, dim[i]);
    }
    if (rep) {
        rep->isolevel_used = iso;
        rep->vmin = mn;
        rep->vmax = mx;
        for (int i = 0; i < 3; i++) { rep->lo[i] = P.lo[i]; rep->hi[i] = P.hi[i]; }
    }
    return N2M_OK;
}

// stage 4: marching cubes into pts_raw / tris_raw
n2m_status march(n2m_context *c, const Prep &P, const int dim[3], int cubes, int *nv_out, int *nt_out,
                 int *ncand_out) {
    c->fwd.valid = false;
    const bool old = cubes == N2M_CUBES_OLDCUBES;
    McGrid g;
    g.vol = P.vol;
    for (int i = 0; i < 3; i++) {
        g.dim[i] = dim[i];
        g.lo[i] = P.lo[i];
        g.n[i] = P.hi[i] - P.lo[i] + 1;
    }
    g.iso = P.iso;
    g.edge_max = P.edge_max;
    volatile float pv = P.mnp - P.iso;
    g.pad_val = pv;
    const double ng = (double)g.n[0] * g.n[1] * g.n[2];
    if (ng >= 4294967040.0) {
        n2m_set_error("grid of %.0f points exceeds the 32-bit range", ng);
        return N2M_ERR_TOO_LARGE;
    }
    CKS(c->totals.ensure(sizeof(uint4)));
    uint4 *dtot = c->totals.as<uint4>();
    if (P.od) {
        const size_t n = (size_t)dim[0] * dim[1] * dim[2];
        CKS(c->stmp2.ensure(n * sizeof(float)));
        const OdRepair rep{P.src, c->stmp.as<float>(), c->stmp2.as<float>(), (float *)P.vol, {dim[0], dim[1], dim[2]},
                           &c->od, &c->scan, P.post};
        if (old) CKS(oc_count(P.vol, dim, P.lo, P.hi, P.iso, P.edge_max, c->mc, c->scan, dtot, c->stream, &rep));
        else CKS(mc_count(g, cubes, c->mc, c->scan, dtot, c->stream, &rep));
    } else if (old) CKS(oc_count(P.vol, dim, P.lo, P.hi, P.iso, P.edge_max, c->mc, c->scan, dtot, c->stream));
    else CKS(mc_count(g, cubes, c->mc, c->scan, dtot, c->stream));
    CK(cudaEventRecord(c->evs[3], c->stream));
    uint4 tot;
    CKS(readback(c, &tot, dtot));
    const unsigned long long nv = (unsigned long long)tot.x + tot.z, nt = tot.y;
    if (nv >= 0x7fffffffULL || nt >= 0x7fffffffULL) {
        n2m_set_error("mesh too large for 32-bit indices");
        return N2M_ERR_TOO_LARGE;
    }
    if ((!old && (nv < 3 || nt < 1)) || (old && nt < 1)) {
        if (old && !g_quiet) printf("marching cubes failed to identify triangles with an isolevel of %g\n", P.iso);
        n2m_set_error("marching cubes produced no surface");
        return N2M_ERR_EMPTY;
    }
    CKS(c->pts_raw.ensure(nv * sizeof(vec3d)));
    CKS(c->tris_raw.ensure(nt * sizeof(vec3i)));
    const int cap = (int)std::min<unsigned long long>(nv / 16 + 65536, 1 << 26);
    CKS(c->cand.ensure((size_t)2 * cap * sizeof(int)));
    CKS(c->ncand.ensure(2 * sizeof(unsigned)));
    CK(cudaMemsetAsync(c->ncand.p, 0, 2 * sizeof(unsigned), c->stream));
    McCounts mcn{tot.x, tot.y, tot.z, tot.w};
    if (old) {
        CKS(oc_emit(P.vol, dim, P.lo, P.hi, P.iso, P.edge_max, c->mc, mcn, c->pts_raw.as<vec3d>(),
                    c->tris_raw.as<vec3i>(), c->cand.as<int>(), c->ncand.as<unsigned>(), cap, c->stream));
    } else {
        CKS(mc_emit(g, cubes, c->mc, mcn, c->pts_raw.as<vec3d>(), c->tris_raw.as<vec3i>(), c->cand.as<int>(),
                    c->ncand.as<unsigned>(), cap, c->stream));
    }
    unsigned nc[2];
    CKS(readback(c, nc, c->ncand.p, 2));
    if (nc[0] > (unsigned)cap || nc[1] > (unsigned)cap) {
        n2m_set_error("weld candidate overflow (%u, %u > %d)", nc[0], nc[1], cap);
        return N2M_ERR_INTERNAL;
    }
    if (nc[1]) {   // c-vertex candidates: collect every vertex near them
        CK(cudaMemcpyAsync(c->cand.as<int>() + nc[0], c->cand.as<int>() + cap, nc[1] * sizeof(int),
                           cudaMemcpyDeviceToDevice, c->stream));
        unsigned tot2 = nc[0] + nc[1];
        CK(cudaMemcpyAsync(c->ncand.p, &tot2, sizeof(unsigned), cudaMemcpyHostToDevice, c->stream));
        CKS(mc_ccand_scan(c->pts_raw.as<vec3d>(), (int)nv, c->cand.as<int>() + cap, (int)nc[1], c->cand.as<int>(),
                          c->ncand.as<unsigned>(), cap, c->stream));
        CKS(readback(c, nc, c->ncand.p, 1));
        if (nc[0] > (unsigned)cap) {
            n2m_set_error("weld candidate overflow");
            return N2M_ERR_INTERNAL;
        }
    }
    CK(cudaEventRecord(c->evs[4], c->stream));
    c->fwd.g = g;
    c->fwd.mcn = mcn;
    c->fwd.cubes = cubes;
    c->fwd.nv_raw = (int)nv;
    *nv_out = (int)nv;
    *nt_out = (int)nt;
    *ncand_out = (int)nc[0];
    return N2M_OK;
}

// the whole meshify on device input; result in c->res_*
n2m_status pipeline(n2m_context *c, const float *d_src, const int dim[3], const n2m_options &o, n2m_report *rep) {
    // no adjoint of an earlier call once this one has started: it may re-allocate what that one used
    c->fwd.valid = false;
    c->res_pts = nullptr;
    c->res_tris = nullptr;
    c->res_np = c->res_nt = 0;
    if (!d_src || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) {
        n2m_set_error("bad volume arguments");
        return N2M_ERR_BAD_ARGS;
    }
    if ((double)dim[0] * dim[1] * dim[2] > 2147483647.0) {
        n2m_set_error("volume exceeds 2^31-1 voxels");
        return N2M_ERR_TOO_LARGE;
    }
    const long long launches0 = g_n2m_launches.load();
    CK(cudaEventRecord(c->ev0, c->stream));
    Prep P;
    CKS(prepare(c, d_src, dim, o, o.verbose, P, rep));
    int nv, nt, ncand;
    CKS(march(c, P, dim, o.cubes, &nv, &nt, &ncand));
    if (c->want_host && !c->user_p) {   // keep buffers started early if they are large enough, else start them now
        const size_t pb = (size_t)std::max(nv, 1) * sizeof(vec3d), tb = (size_t)std::max(nt, 1) * sizeof(vec3i);
        if (!c->hout.pts || c->hout.pb < pb || c->hout.tb < tb) c->hout.start(pb, tb);
        c->hint_pb = pb;
        c->hint_tb = tb;
    }
    vec3d *pts = c->pts_raw.as<vec3d>();
    int np = nv;
    int welded = 0;
    c->fwd.nrem = c->fwd.nov = 0;
    if (ncand > 0) {
        std::vector<int> removed, keep, ov_id, ov_src;
        std::vector<vec3d> ov_pos;
        std::vector<int2> corners;
        if (o.cubes == N2M_CUBES_OLDCUBES) {
            CKS(weld_oc(c, P, dim, nv, nt, ncand, removed, keep, ov_id, ov_pos, ov_src, corners));
        } else {
            vec3d v0;
            CKS(readback(c, &v0, pts));
            CKS(weld_candidates(c, nv, ncand, removed, keep, ov_id, ov_pos, ov_src, v0));
        }
        if (!removed.empty() || !ov_id.empty()) {
            const int nr = (int)removed.size(), no = (int)ov_id.size(), ncr = (int)corners.size();
            CKS(c->weld.ensure((size_t)(2 * nr + 2 * no + 2) * sizeof(int) + (size_t)(no + 1) * sizeof(vec3d) +
                               (size_t)(ncr + 1) * sizeof(int2)));
            vec3d *dov = c->weld.as<vec3d>();
            int2 *dcr = (int2 *)(dov + no + 1);
            int *drem = (int *)(dcr + ncr + 1);
            int *dkeep = drem + nr, *dovid = dkeep + nr, *dovsrc = dovid + no + 1;
            if (no) CK(cudaMemcpyAsync(dov, ov_pos.data(), no * sizeof(vec3d), cudaMemcpyHostToDevice, c->stream));
            if (nr) CK(cudaMemcpyAsync(drem, removed.data(), nr * sizeof(int), cudaMemcpyHostToDevice, c->stream));
            if (nr) CK(cudaMemcpyAsync(dkeep, keep.data(), nr * sizeof(int), cudaMemcpyHostToDevice, c->stream));
            if (no) CK(cudaMemcpyAsync(dovid, ov_id.data(), no * sizeof(int), cudaMemcpyHostToDevice, c->stream));
            if (no) CK(cudaMemcpyAsync(dovsrc, ov_src.data(), no * sizeof(int), cudaMemcpyHostToDevice, c->stream));
            if (ncr) {   // split vertices: corners take their copy's group vertex before the renumbering
                CK(cudaMemcpyAsync(dcr, corners.data(), ncr * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
                { k_set_corners<<<(ncr + 255) / 256, 256, 0, c->stream>>>(c->tris_raw.as<vec3i>(), dcr, ncr); N2M_COUNT(); }
                CKL();
            }
            c->fwd.removed = drem;
            c->fwd.ov_id = dovid;
            c->fwd.ov_src = dovsrc;
            c->fwd.nrem = nr;
            c->fwd.nov = no;
            np = nv - nr;
            CKS(c->pts.ensure((size_t)np * sizeof(vec3d)));
            CKS(mesh_apply_weld(pts, c->tris_raw.as<vec3i>(), nv, nt, drem, dkeep, nr, dovid, dov, no,
                                c->pts.as<vec3d>(), c->stream));
            pts = c->pts.as<vec3d>();
            welded = nr;
            CK(cudaStreamSynchronize(c->stream));   // host vectors go out of scope
        }
    }
    CK(cudaEventRecord(c->evs[5], c->stream));
    if (np < 3) {
        n2m_set_error("fewer than 3 vertices after the weld");
        return N2M_ERR_EMPTY;
    }
    CKS(c->tris.ensure((size_t)nt * sizeof(vec3i)));
    CKS(c->ntf.ensure(sizeof(unsigned)));
    c->pts_early = false;
    const bool early = c->want_host && o.post_smooth <= 0;   // vertices are final after the weld
    if (early) CK(cudaEventRecord(c->stage.ev[0], c->stream));
    CKS(mesh_remove_degenerate(pts, c->tris_raw.as<vec3i>(), nt, c->tris.as<vec3i>(), c->ntf.as<unsigned>(), c->deg,
                               c->scan, c->stream));
    if (early) {   // copy them out on the second stream while the degenerate filter runs
        void *dst = nullptr;
        if (c->user_p) {
            if ((size_t)np <= c->user_pcap) dst = c->user_p;
        } else {
            c->hout.join();
            if (c->hout.pts && c->hout.pb >= (size_t)np * sizeof(vec3d)) dst = c->hout.pts;
        }
        if (dst) {
            CK(cudaStreamWaitEvent(c->copy, c->stage.ev[0], 0));
            CK(cudaMemcpyAsync(dst, pts, (size_t)np * sizeof(vec3d), cudaMemcpyDeviceToHost, c->copy));
            c->pts_early = true;
        }
    }
    CK(cudaEventRecord(c->evs[6], c->stream));
    CK(cudaEventRecord(c->ev1, c->stream));
    unsigned ntf;
    CKS(readback(c, &ntf, c->ntf.p));
    c->res_pts = pts;
    c->res_tris = c->tris.as<vec3i>();
    c->res_np = np;
    c->res_nt = (int)ntf;
    c->fwd.valid = true;
    c->fwd.smoothed = o.pre_smooth && dim[0] >= 5 && dim[1] >= 5 && dim[2] >= 5;
    c->fwd.clustered = o.only_largest || o.fill_bubbles;
    c->fwd.post_smooth = 0;
    for (int i = 0; i < 3; i++) c->fwd.dim[i] = dim[i];
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (o.verbose) {
        printf("marching cubes (%dx%dx%d) + weld + degenerate removal on GPU: %.3f ms\n", dim[0], dim[1], dim[2], ms);
        if (welded) printf("vertex welding %d -> %d\n", nv, np);
        if ((int)ntf != nt) printf("remove degenerate triangles %d -> %u\n", nt, ntf);
    }
    if (rep) {
        rep->nvert_raw = nv;
        rep->ntri_raw = nt;
        rep->nvert = np;
        rep->ntri = ntf;
        rep->welded = welded;
        rep->degenerate = nt - (int)ntf;
        rep->ms_total = ms;
        for (int i = 0; i < 6; i++) {
            rep->ms_stage[i] = 0.f;
            cudaEventElapsedTime(&rep->ms_stage[i], c->evs[i], c->evs[i + 1]);
        }
        rep->ms_stage[6] = rep->ms_stage[7] = 0.f;
        rep->kernel_launches = g_n2m_launches.load() - launches0;
        rep->ms_smooth_pass_a = 0.f;
        if (c->pass_a) cudaEventElapsedTime(&rep->ms_smooth_pass_a, c->eva[0], c->eva[1]);
    }
    return N2M_OK;
}

n2m_status to_host_mesh(n2m_context *c, vec3i **t, vec3d **p, int *nt, int *np, n2m_report *rep = nullptr) {
    const auto t0 = std::chrono::steady_clock::now();
    const size_t pbytes = (size_t)c->res_np * sizeof(vec3d), tbytes = (size_t)std::max(c->res_nt, 1) * sizeof(vec3i);
    c->hout.join();
    bool early = c->pts_early;   // final vertices already copied into hout.pts on the second stream
    c->pts_early = false;
    if (early) CK(cudaStreamSynchronize(c->copy));
    vec3d *hp;
    vec3i *ht;
    if (c->hout.pts && c->hout.pb >= pbytes && c->hout.tb >= tbytes) {   // pre-faulted (sized for the raw mesh)
        hp = (vec3d *)c->hout.pts;
        ht = (vec3i *)c->hout.tris;
        c->hout.pts = c->hout.tris = nullptr;
        c->hout.pb = c->hout.tb = 0;
    } else {
        early = false;
        c->hout.discard();
        hp = (vec3d *)malloc(std::max<size_t>(pbytes, 1));
        ht = (vec3i *)malloc(tbytes);
        if (!hp || !ht) {
            free(hp);
            free(ht);
            n2m_set_error("host allocation failed");
            return N2M_ERR_OOM;
        }
    }
    cudaError_t e = early ? cudaSuccess : cudaMemcpyAsync(hp, c->res_pts, pbytes, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ht, c->res_tris, (size_t)c->res_nt * sizeof(vec3i), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        free(hp);
        free(ht);
        n2m_set_error("mesh readback: %s", cudaGetErrorString(e));
        return N2M_ERR_CUDA;
    }
    *t = ht;
    *p = hp;
    *nt = c->res_nt;
    *np = c->res_np;
    if (rep) rep->ms_stage[7] = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return N2M_OK;
}

// the mesh into the caller's buffers (n2m_meshify_into)
n2m_status to_user_mesh(n2m_context *c, int *nt, int *np, n2m_report *rep) {
    const auto t0 = std::chrono::steady_clock::now();
    const bool early = c->pts_early;
    c->pts_early = false;
    if (early) CK(cudaStreamSynchronize(c->copy));
    *nt = c->res_nt;
    *np = c->res_np;
    if ((size_t)c->res_nt > c->user_tcap || (size_t)c->res_np > c->user_pcap) {
        n2m_set_error("mesh of %d triangles and %d vertices does not fit the output buffers (%zu, %zu)", c->res_nt,
                      c->res_np, c->user_tcap, c->user_pcap);
        return N2M_ERR_TOO_LARGE;
    }
    if (!early && c->res_np)
        CK(cudaMemcpyAsync(c->user_p, c->res_pts, (size_t)c->res_np * sizeof(vec3d), cudaMemcpyDeviceToHost, c->stream));
    if (c->res_nt)
        CK(cudaMemcpyAsync(c->user_t, c->res_tris, (size_t)c->res_nt * sizeof(vec3i), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    if (rep) rep->ms_stage[7] = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return N2M_OK;
}

n2m_status upload(n2m_context *c, const float *img, size_t n) {
    CKS(c->in.ensure(n * sizeof(float)));
    CK(cudaMemcpyAsync(c->in.p, img, n * sizeof(float), cudaMemcpyHostToDevice, c->stream));
    return N2M_OK;
}
}  // namespace

// ---- explicit-status API -------------------------------------------------------------
extern "C" n2m_status n2m_meshify_device(n2m_context *c, const float *d_img, const int dim[3], const n2m_options *opt,
                                         vec3i **d_t, vec3d **d_p, int *nt, int *np, n2m_report *rep) {
    if (!c || !opt || !dim) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    CKS(pipeline(c, d_img, dim, *opt, rep));
    c->fwd.post_smooth = opt->post_smooth > 0 ? opt->post_smooth : 0;
    if (opt->post_smooth > 0) {
        const long long l0 = g_n2m_launches.load();
        CK(cudaEventRecord(c->evs[6], c->stream));
        CKS(mesh_smooth_hc(c->res_pts, c->res_tris, c->res_np, c->res_nt, 0.1, 0.5, opt->post_smooth, true, c->hc,
                           c->scan, c->stream));
        CK(cudaEventRecord(c->evs[7], c->stream));
        CK(cudaStreamSynchronize(c->stream));
        if (rep) {
            cudaEventElapsedTime(&rep->ms_stage[6], c->evs[6], c->evs[7]);
            rep->kernel_launches += g_n2m_launches.load() - l0;
        }
    }
    CK(cudaStreamSynchronize(c->stream));
    if (d_t) *d_t = c->res_tris;
    if (d_p) *d_p = c->res_pts;
    if (nt) *nt = c->res_nt;
    if (np) *np = c->res_np;
    return N2M_OK;
}

namespace {
// pipeline on c->in (filled or being filled by a staged upload), HC, and the
// mesh into pre-faulted malloc memory; on failure no copy may still read the
// caller's volume and no output buffer is kept
n2m_status meshify_host_tail(n2m_context *c, const int dim[3], const n2m_options *opt, vec3i **t, vec3d **p, int *nt,
                             int *np, n2m_report *rep) {
    c->want_host = true;
    // fault in output pages sized like the last call's mesh while the GPU works (re-sized after the count if short)
    if (c->hint_pb && !c->user_p) c->hout.start(c->hint_pb + c->hint_pb / 8, c->hint_tb + c->hint_tb / 8);
    n2m_status s = pipeline(c, c->in.as<float>(), dim, *opt, rep);
    c->stage.host = nullptr;
    c->want_host = false;
    c->fwd.post_smooth = opt->post_smooth > 0 ? opt->post_smooth : 0;
    if (s == N2M_OK && opt->post_smooth > 0)
        s = mesh_smooth_hc(c->res_pts, c->res_tris, c->res_np, c->res_nt, 0.1, 0.5, opt->post_smooth, true, c->hc, c->scan,
                           c->stream);
    if (s == N2M_OK) s = c->user_p ? to_user_mesh(c, nt, np, rep) : to_host_mesh(c, t, p, nt, np, rep);
    if (s != N2M_OK) {
        cudaStreamSynchronize(c->copy);
        c->pts_early = false;
        c->hout.discard();
    }
    return s;
}

// host volume in (staged upload when pre-smoothing), mesh out through meshify_host_tail
n2m_status meshify_host(n2m_context *c, const float *img, const int dim[3], const n2m_options *opt, vec3i **t,
                        vec3d **p, int *nt, int *np, n2m_report *rep) {
    const size_t n = (size_t)dim[0] * dim[1] * dim[2];
    // with pre-smoothing the upload is staged: the x pass of each slab starts as soon as it has arrived
    const bool staged = opt->pre_smooth && dim[0] >= 5 && dim[1] >= 5 && dim[2] >= 5 && smooth_can_stage(dim[0], dim[1], dim[2]);
    if (staged) {
        CKS(c->in.ensure(n * sizeof(float)));
        c->stage.host = img;
    } else {
        CKS(upload(c, img, n));
    }
    return meshify_host_tail(c, dim, opt, t, p, nt, np, rep);
}
}  // namespace

extern "C" n2m_status n2m_meshify(n2m_context *c, const float *img, const int dim[3], const n2m_options *opt,
                                  vec3i **t, vec3d **p, int *nt, int *np, n2m_report *rep) {
    if (!c || !opt || !dim || !img || !t || !p || !nt || !np) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    return meshify_host(c, img, dim, opt, t, p, nt, np, rep);
}

extern "C" n2m_status n2m_meshify_into(n2m_context *c, const float *img, const int dim[3], const n2m_options *opt,
                                       vec3i *t, int64_t t_cap, vec3d *p, int64_t p_cap, int *nt, int *np,
                                       n2m_report *rep) {
    if (!c || !opt || !dim || !img || !nt || !np || t_cap < 0 || p_cap < 0 || (t_cap && !t) || (p_cap && !p))
        return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    static vec3d no_pts;   // a non-null marker when the caller passes no vertex space
    c->user_t = t;
    c->user_p = p ? p : &no_pts;
    c->user_tcap = (size_t)t_cap;
    c->user_pcap = p ? (size_t)p_cap : 0;
    const n2m_status s = meshify_host(c, img, dim, opt, nullptr, nullptr, nt, np, rep);
    c->user_t = nullptr;
    c->user_p = nullptr;
    c->user_tcap = c->user_pcap = 0;
    return s;
}

extern "C" n2m_status n2m_cast_voxels_device(n2m_context *c, const void *d_raw, int datatype, float scl_slope,
                                             float scl_inter, int64_t nvox, float *d_out) {
    if (!c || (nvox > 0 && (!d_raw || !d_out))) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    CKS(launch_cast(d_raw, datatype, scl_slope, scl_inter, nvox, d_out, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return N2M_OK;
}

extern "C" n2m_status n2m_meshify_typed(n2m_context *c, const void *img, int datatype, float scl_slope, float scl_inter,
                                        const int dim[3], const n2m_options *opt, vec3i **t, vec3d **p, int *nt,
                                        int *np, n2m_report *rep) {
    if (!c || !opt || !dim || !img || !t || !p || !nt || !np) return N2M_ERR_BAD_ARGS;
    const int bpp = nifti_bytes_per_voxel(datatype);
    if (!bpp) {
        n2m_set_error("unsupported NIfTI datatype %d (uint8 2, int16 4, float32 16, uint16 512)", datatype);
        return N2M_ERR_BAD_ARGS;
    }
    if (dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    c->hout.discard();
    const size_t nxy = (size_t)dim[0] * dim[1], n = nxy * dim[2];
    CKS(c->raw.ensure(n * bpp));
    CKS(c->in.ensure(n * sizeof(float)));
    // raw slabs on the copy stream; each is cast on the main stream as soon as it has arrived
    CK(cudaEventRecord(c->stage.ev[N2M_STAGE_SLABS], c->stream));
    CK(cudaStreamWaitEvent(c->copy, c->stage.ev[N2M_STAGE_SLABS], 0));
    n2m_status s = N2M_OK;
    for (int k = 0; k < N2M_STAGE_SLABS && s == N2M_OK; k++) {
        const size_t z0 = (size_t)dim[2] * k / N2M_STAGE_SLABS, z1 = (size_t)dim[2] * (k + 1) / N2M_STAGE_SLABS;
        if (z1 <= z0) continue;
        const size_t off = z0 * nxy, cnt = (z1 - z0) * nxy;
        if (cudaMemcpyAsync((char *)c->raw.p + off * bpp, (const char *)img + off * bpp, cnt * bpp, cudaMemcpyHostToDevice,
                            c->copy) != cudaSuccess ||
            cudaEventRecord(c->stage.ev[k], c->copy) != cudaSuccess ||
            cudaStreamWaitEvent(c->stream, c->stage.ev[k], 0) != cudaSuccess) {
            n2m_set_error("staged upload: %s", cudaGetErrorString(cudaGetLastError()));
            s = N2M_ERR_CUDA;
            break;
        }
        s = launch_cast((const char *)c->raw.p + off * bpp, datatype, scl_slope, scl_inter, (long long)cnt,
                        c->in.as<float>() + off, c->stream);
    }
    if (s != N2M_OK) {
        cudaStreamSynchronize(c->copy);
        return s;
    }
    return meshify_host_tail(c, dim, opt, t, p, nt, np, rep);
}

extern "C" n2m_status n2m_meshify_backward(n2m_context *c, const float *d_grad_pts, float *d_grad_img) {
    if (!c || !d_grad_pts || !d_grad_img) return N2M_ERR_BAD_ARGS;
    if (!c->fwd.valid) {
        n2m_set_error("n2m_meshify_backward: no forward pass on this context");
        return N2M_ERR_BAD_ARGS;
    }
    if (c->fwd.clustered || c->fwd.cubes == N2M_CUBES_OLDCUBES) {
        n2m_set_error("n2m_meshify_backward: supported for the Lewiner cubes without clustering (-l 0 -b 0)");
        return N2M_ERR_BAD_ARGS;
    }
    CK(cudaSetDevice(c->device));
    const int np = c->res_np, nvr = c->fwd.nv_raw;
    const size_t nvox = (size_t)c->fwd.dim[0] * c->fwd.dim[1] * c->fwd.dim[2];
    CKS(c->gA.ensure((size_t)np * sizeof(float3)));
    CKS(c->gB.ensure((size_t)nvr * sizeof(float3)));
    CKS(c->gs.ensure(nvox * sizeof(float)));
    const float3 *go = (const float3 *)d_grad_pts;
    if (c->fwd.post_smooth > 0) {
        CKS(mesh_smooth_hc_backward(c->res_tris, np, 0.1, 0.5, c->fwd.post_smooth, true, c->hc, go, c->gA.as<float3>(),
                                    c->stream));
        go = c->gA.as<float3>();
    }
    const float3 *graw = go;
    if (c->fwd.nrem > 0) {
        CKS(mesh_weld_backward(go, np, nvr, c->fwd.removed, c->fwd.nrem, c->fwd.ov_id, c->fwd.ov_src, c->fwd.nov,
                               c->gB.as<float3>(), c->stream));
        graw = c->gB.as<float3>();
    }
    float *gs = c->fwd.smoothed ? c->gs.as<float>() : d_grad_img;
    CK(cudaMemsetAsync(gs, 0, nvox * sizeof(float), c->stream));
    CKS(mc_backward(c->fwd.g, c->fwd.cubes, c->mc, c->fwd.mcn, graw, gs, c->stream));
    if (c->fwd.smoothed) {
        CKS(c->gtmp.ensure(nvox * sizeof(float)));
        CKS(launch_smooth_adjoint(gs, c->gtmp.as<float>(), d_grad_img, c->fwd.dim[0], c->fwd.dim[1], c->fwd.dim[2],
                                  c->stream));
    }
    CK(cudaStreamSynchronize(c->stream));
    return N2M_OK;
}

extern "C" n2m_status n2m_smooth_hc_device(n2m_context *c, vec3d *d_verts, const vec3i *d_tris, int nvert, int ntri,
                                           double alpha, double beta, int iter, bool lock_edges) {
    if (!c) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    if (nvert < 0 || ntri < 0) return N2M_ERR_BAD_ARGS;
    CKS(mesh_smooth_hc(d_verts, d_tris, nvert, ntri, alpha, beta, iter, lock_edges, c->hc, c->scan, c->stream));
    CKS(mesh_smooth_hc_check(c->hc, nvert, iter, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return N2M_OK;
}


// ---- atlas ---------------------------------------------------------------------------
namespace {
n2m_status atlas_loop(n2m_context *c, const int16_t *d_lab, const int dim[3], const n2m_options &opt,
                      int64_t *npts, int64_t *ntris) {
    int maxlab = 0;
    std::vector<unsigned> cnt;
    std::vector<int> bb;
    CKS(atlas_hist((const short *)d_lab, dim, c->aw, c->stream, &maxlab, cnt, bb));
    if (maxlab < 1) {
        n2m_set_error("intensity range not consistent with an indexed atlas");
        return N2M_ERR_BAD_ARGS;
    }
    const long long n = (long long)dim[0] * dim[1] * dim[2];
    CKS(c->in.ensure((size_t)n * sizeof(float)));
    n2m_options o = opt;
    o.isolevel = 0.5f;
    o.verbose = false;
    int64_t vp = 0, tp = 0;
    for (int l = 1; l <= maxlab; l++) {
        if (!cnt[l]) continue;   // "Skipping %d: no voxels with this intensity" (src/nii2mesh.c:565)
        CKS(atlas_binarize((const short *)d_lab, n, l, c->in.as<float>(), c->stream));
        n2m_atlas_mesh d = {l, N2M_OK, 0, 0, vp, tp};
        const n2m_status st = pipeline(c, c->in.as<float>(), dim, o, nullptr);
        if (st == N2M_ERR_NO_VARIABILITY || st == N2M_ERR_EMPTY) {
            d.status = st;
            c->atlas_meshes.push_back(d);
            continue;
        }
        CKS(st);
        if (o.post_smooth > 0)
            CKS(mesh_smooth_hc(c->res_pts, c->res_tris, c->res_np, c->res_nt, 0.1, 0.5, o.post_smooth, true, c->hc,
                               c->scan, c->stream));
        const size_t needp = (size_t)(vp + c->res_np) * sizeof(vec3d), needt = (size_t)(tp + c->res_nt) * sizeof(vec3i);
        for (int k = 0; k < 2; k++) {   // grow the concatenated outputs, keeping what they hold
            DevBuf &B = k ? c->ltris : c->lpts;
            const size_t need = k ? needt : needp, used = k ? (size_t)tp * sizeof(vec3i) : (size_t)vp * sizeof(vec3d);
            if (need > B.cap) {
                DevBuf nb;
                CKS(nb.ensure(std::max(need, 2 * B.cap)));
                if (used) CK(cudaMemcpyAsync(nb.p, B.p, used, cudaMemcpyDeviceToDevice, c->stream));
                CK(cudaStreamSynchronize(c->stream));
                B.release();
                B = nb;
            }
        }
        CK(cudaMemcpyAsync(c->lpts.as<vec3d>() + vp, c->res_pts, (size_t)c->res_np * sizeof(vec3d),
                           cudaMemcpyDeviceToDevice, c->stream));
        CK(cudaMemcpyAsync(c->ltris.as<vec3i>() + tp, c->res_tris, (size_t)c->res_nt * sizeof(vec3i),
                           cudaMemcpyDeviceToDevice, c->stream));
        d.nvert = c->res_np;
        d.ntri = c->res_nt;
        c->atlas_meshes.push_back(d);
        vp += c->res_np;
        tp += c->res_nt;
    }
    CK(cudaStreamSynchronize(c->stream));
    *npts = vp;
    *ntris = tp;
    return N2M_OK;
}
}  // namespace

extern "C" n2m_status n2m_atlas_device(n2m_context *c, const int16_t *d_labels, const int dim[3], const n2m_options *opt,
                                       int mode, int *nmesh, const n2m_atlas_mesh **meshes, vec3d **d_pts,
                                       vec3i **d_tris, int64_t *npts, int64_t *ntris, n2m_report *rep) {
    if (!c || !d_labels || !dim || !opt || dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) return N2M_ERR_BAD_ARGS;
    if (opt->cubes == N2M_CUBES_OLDCUBES) {
        n2m_set_error("n2m_atlas: the batched atlas supports the Lewiner cubes");
        return N2M_ERR_BAD_ARGS;
    }
    CK(cudaSetDevice(c->device));
    struct Quiet {
        Quiet() { g_quiet = true; }
        ~Quiet() { g_quiet = false; }
    } quiet;
    c->fwd.valid = false;
    c->atlas_meshes.clear();
    const long long l0 = g_n2m_launches.load();
    CK(cudaEventRecord(c->ev0, c->stream));
    int64_t np = 0, nt = 0;
    vec3d *pp = nullptr;
    vec3i *tt = nullptr;
    float stage[8] = {0};
    if (mode == N2M_ATLAS_LOOP) {
        CKS(atlas_loop(c, d_labels, dim, *opt, &np, &nt));
        pp = c->lpts.as<vec3d>();
        tt = c->ltris.as<vec3i>();
    } else {
        CKS(atlas_batched((const short *)d_labels, dim, *opt, c->aw, c->scan, c->deg, c->hc, c->stream, c->atlas_meshes,
                          &pp, &tt, &np, &nt, stage));
    }
    CK(cudaEventRecord(c->ev1, c->stream));
    CK(cudaEventSynchronize(c->ev1));
    if (rep) {
        memset(rep, 0, sizeof(*rep));
        cudaEventElapsedTime(&rep->ms_total, c->ev0, c->ev1);
        for (int i = 0; i < 8; i++) rep->ms_stage[i] = stage[i];
        rep->nvert = np;
        rep->ntri = nt;
        rep->kernel_launches = g_n2m_launches.load() - l0;
    }
    if (nmesh) *nmesh = (int)c->atlas_meshes.size();
    if (meshes) *meshes = c->atlas_meshes.data();
    if (d_pts) *d_pts = pp;
    if (d_tris) *d_tris = tt;
    if (npts) *npts = np;
    if (ntris) *ntris = nt;
    return N2M_OK;
}

extern "C" n2m_status n2m_atlas(n2m_context *c, const int16_t *labels, const int dim[3], const n2m_options *opt, int mode,
                                int *nmesh, n2m_atlas_mesh **meshes, vec3d **pts, vec3i **tris, int64_t *npts,
                                int64_t *ntris) {
    if (!c || !labels || !dim || !nmesh || !meshes || !pts || !tris || !npts || !ntris) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    const size_t n = (size_t)dim[0] * dim[1] * dim[2];
    CKS(c->alab.ensure(n * sizeof(int16_t)));
    CK(cudaMemcpyAsync(c->alab.p, labels, n * sizeof(int16_t), cudaMemcpyHostToDevice, c->stream));
    const n2m_atlas_mesh *dm;
    vec3d *dp;
    vec3i *dt;
    int nm;
    CKS(n2m_atlas_device(c, c->alab.as<int16_t>(), dim, opt, mode, &nm, &dm, &dp, &dt, npts, ntris, nullptr));
    *meshes = (n2m_atlas_mesh *)malloc(std::max(nm, 1) * sizeof(n2m_atlas_mesh));
    *pts = (vec3d *)malloc(std::max<int64_t>(*npts, 1) * sizeof(vec3d));
    *tris = (vec3i *)malloc(std::max<int64_t>(*ntris, 1) * sizeof(vec3i));
    if (!*meshes || !*pts || !*tris) {
        free(*meshes); free(*pts); free(*tris);
        n2m_set_error("host allocation failed");
        return N2M_ERR_OOM;
    }
    memcpy(*meshes, dm, nm * sizeof(n2m_atlas_mesh));
    *nmesh = nm;
    CK(cudaMemcpyAsync(*pts, dp, (size_t)*npts * sizeof(vec3d), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(*tris, dt, (size_t)*ntris * sizeof(vec3i), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    return N2M_OK;
}

// ---- drop-in entry points ---------------------------------------------------------------
static void report_failure(const char *fn, n2m_status s) {
    if (s == N2M_ERR_NO_VARIABILITY || s == N2M_ERR_EMPTY) return;   // reference prints its own message
    printf("%s: %s (%s)\n", fn, n2m_status_string(s), n2m_last_error());
}

extern "C" int n2m_set_oldcubes(int enable) {
    const int old = g_oldcubes;
    g_oldcubes = enable;
    return old;
}

extern "C" int meshify(float *img, short dim[3], int originalMC, float isolevel, vec3i **t, vec3d **p, int *nt,
                       int *np, bool preSmooth, bool onlyLargest, bool fillBubbles, bool verbose) {
    n2m_context *c;
    n2m_status s = default_ctx(&c);
    if (s == N2M_OK) {
        const int d[3] = {dim[0], dim[1], dim[2]};
        n2m_options o = {g_oldcubes ? (int)N2M_CUBES_OLDCUBES : (originalMC ? (int)N2M_CUBES_CLASSIC_TABLE : (int)N2M_CUBES_MC33),
                         isolevel, preSmooth, onlyLargest, fillBubbles, 0, verbose};
        s = n2m_meshify(c, img, d, &o, t, p, nt, np, nullptr);
    }
    if (s != N2M_OK) {
        report_failure("meshify", s);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

extern "C" void laplacian_smoothHC(vec3d *verts, vec3i *tris, int nvert, int ntri, double alpha, double beta, int iter,
                                   bool lockEdges) {
    n2m_context *c;
    n2m_status s = default_ctx(&c);
    if (s == N2M_OK && (nvert < 0 || ntri < 0 || (nvert > 0 && !verts) || (ntri > 0 && !tris))) {
        n2m_set_error("laplacian_smoothHC: bad arguments");
        s = N2M_ERR_BAD_ARGS;
    }
    if (s == N2M_OK && nvert > 0 && iter > 0) {
        s = N2M_ERR_CUDA;
        if (c->hmesh.ensure((size_t)nvert * sizeof(vec3d) + (size_t)std::max(ntri, 1) * sizeof(vec3i)) == N2M_OK) {
            vec3d *dv = c->hmesh.as<vec3d>();
            vec3i *dt = (vec3i *)(dv + nvert);
            if (cudaMemcpyAsync(dv, verts, (size_t)nvert * sizeof(vec3d), cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
                cudaMemcpyAsync(dt, tris, (size_t)ntri * sizeof(vec3i), cudaMemcpyHostToDevice, c->stream) == cudaSuccess) {
                s = mesh_smooth_hc(dv, dt, nvert, ntri, alpha, beta, iter, lockEdges, c->hc, c->scan, c->stream);
                if (s == N2M_OK) s = mesh_smooth_hc_check(c->hc, nvert, iter, c->stream);
                if (s == N2M_OK &&
                    (cudaMemcpyAsync(verts, dv, (size_t)nvert * sizeof(vec3d), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                     cudaStreamSynchronize(c->stream) != cudaSuccess))
                    s = N2M_ERR_CUDA;
            }
        }
    }
    if (s != N2M_OK) report_failure("laplacian_smoothHC", s);
}

extern "C" n2m_status n2m_set_threshold_device(n2m_context *c, const float *d_img, int64_t nvox, int mode, float *iso) {
    if (!c || !iso || (nvox > 0 && !d_img)) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    return isolevel_otsu(d_img, nvox, mode, c->th, c->stream, iso);
}

extern "C" n2m_status n2m_set_threshold(n2m_context *c, const float *img, int64_t nvox, int mode, float *iso) {
    if (!c || !iso || (nvox > 0 && !img)) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    if (nvox > 0) CKS(upload(c, img, (size_t)nvox));
    return isolevel_otsu(c->in.as<float>(), nvox, mode, c->th, c->stream, iso);
}

extern "C" float setThreshold(float *img, int nvox, int darkMediumBright123) {
    n2m_context *c;
    float iso = 1.0f;
    n2m_status s = default_ctx(&c);
    if (s == N2M_OK) s = n2m_set_threshold(c, img, nvox, darkMediumBright123, &iso);
    if (s != N2M_OK) report_failure("setThreshold", s);
    return iso;
}

extern "C" void apply_sform(vec3i *t, vec3d *p, int nt, int np, float srow_x[4], float srow_y[4], float srow_z[4]) {
    n2m_context *c;
    n2m_status s = default_ctx(&c);
    if (s == N2M_OK && np > 0) {
        s = N2M_ERR_CUDA;
        if (c->hmesh.ensure((size_t)np * sizeof(vec3d) + (size_t)std::max(nt, 1) * sizeof(vec3i)) == N2M_OK) {
            vec3d *dv = c->hmesh.as<vec3d>();
            vec3i *dt = (vec3i *)(dv + np);
            if (cudaMemcpyAsync(dv, p, (size_t)np * sizeof(vec3d), cudaMemcpyHostToDevice, c->stream) == cudaSuccess &&
                cudaMemcpyAsync(dt, t, (size_t)nt * sizeof(vec3i), cudaMemcpyHostToDevice, c->stream) == cudaSuccess) {
                s = mesh_apply_sform(dv, dt, np, nt, srow_x, srow_y, srow_z, c->stream);
                if (s == N2M_OK &&
                    (cudaMemcpyAsync(p, dv, (size_t)np * sizeof(vec3d), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                     cudaMemcpyAsync(t, dt, (size_t)nt * sizeof(vec3i), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                     cudaStreamSynchronize(c->stream) != cudaSuccess))
                    s = N2M_ERR_CUDA;
            }
        }
    }
    if (s != N2M_OK) report_failure("apply_sform", s);
}

extern "C" int bwlabel(float *img, int conn, size_t dim[3], bool onlyLargest, bool fillBubbles) {
    if (conn != 6 && conn != 18 && conn != 26) {
        fprintf(stderr, "bwlabel: conn must be 6, 18 or 26.\n");
        return 0;
    }
    if (dim[0] < 2 || dim[1] < 2 || dim[2] < 1) {
        fprintf(stderr, "bwlabel: img must be 2 or 3-dimensional\n");
        return 0;
    }
    n2m_context *c;
    n2m_status s = default_ctx(&c);
    int nl = 0;
    if (s == N2M_OK) {
        const size_t n = dim[0] * dim[1] * dim[2];
        s = upload(c, img, n);
        if (s == N2M_OK) s = c->ntf.ensure(sizeof(int));
        if (s == N2M_OK)
            s = run_bwlabel(c->in.as<float>(), (int)dim[0], (int)dim[1], (int)dim[2], conn, onlyLargest, fillBubbles,
                            c->lab, c->scan, c->ntf.as<int>(), c->stream);
        if (s == N2M_OK && (cudaMemcpyAsync(img, c->in.p, n * sizeof(float), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess))
            s = N2M_ERR_CUDA;
        if (s == N2M_OK) s = readback(c, &nl, c->ntf.p);
    }
    if (s != N2M_OK) {
        report_failure("bwlabel", s);
        return 0;
    }
    return nl;
}

extern "C" int marchingCubes(float *img, short dim[3], int lo[3], int hi[3], int originalMC, float isolevel,
                             vec3d **vs, vec3i **ts, int *nv, int *nt) {
    n2m_context *c;
    n2m_status s = default_ctx(&c);
    if (s == N2M_OK) {
        const int d[3] = {dim[0], dim[1], dim[2]};
        const size_t n = (size_t)d[0] * d[1] * d[2];
        s = upload(c, img, n);
        Prep P;
        P.vol = c->in.as<float>();
        P.iso = isolevel;
        P.edge_max = INFINITY;   // the standalone call does not darken edges
        for (int i = 0; i < 3; i++) { P.lo[i] = lo[i]; P.hi[i] = hi[i]; }
        if (s == N2M_OK) {   // padding: min of the whole volume (src/MarchingCubes.c:1094-1098)
            CKS(c->stats.ensure(sizeof(VolStats)));
            VolStats h;
            stats_init_host(&h);
            if (cudaMemcpyAsync(c->stats.p, &h, sizeof(h), cudaMemcpyHostToDevice, c->stream) != cudaSuccess) s = N2M_ERR_CUDA;
            if (s == N2M_OK) s = launch_stats(P.vol, d[0], d[1], d[2], isolevel, true, c->stats.as<VolStats>(), c->stream);
            if (s == N2M_OK) s = readback(c, &h, c->stats.p);
            P.mnp = ord2f(h.vmin);
        }
        const int cubes = g_oldcubes ? N2M_CUBES_OLDCUBES : (originalMC ? N2M_CUBES_CLASSIC_TABLE : N2M_CUBES_MC33);
        int v = 0, t = 0, ncand = 0;
        if (s == N2M_OK) s = march(c, P, d, cubes, &v, &t, &ncand);
        if (s == N2M_OK) {
            c->res_pts = c->pts_raw.as<vec3d>();
            c->res_tris = c->tris_raw.as<vec3i>();
            c->res_np = v;
            c->res_nt = t;
            s = to_host_mesh(c, ts, vs, nt, nv);
        }
    }
    if (s != N2M_OK) {
        report_failure("marchingCubes", s);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

// ---- mesh writers ------------------------------------------------------------------------------
extern "C" int n2m_mesh_format_of(const char *fnm) { return fnm ? mesh_format_of(fnm) : -1; }

// ---- the rest of meshify.h ----------------------------------------------------------------------
extern "C" void strip_ext(char *fname) {
    if (fname) fname[file_ext(fname) - fname] = '\0';
}

extern "C" double clockMsec(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec * 1000.0 + t.tv_nsec / 1.0e6;
}

extern "C" long timediff(double startTimeMsec, double endTimeMsec) { return lround(endTimeMsec - startTimeMsec); }

namespace {
// host mesh -> context buffers (vertices after the triangles, 8-byte aligned)
n2m_status upload_mesh(n2m_context *c, const vec3i *tris, const vec3d *pts, int nt, int np, const vec3i **dt,
                       const vec3d **dp) {
    if (nt < 0 || np < 0 || (nt && !tris) || (np && !pts)) return N2M_ERR_BAD_ARGS;
    CKS(c->wr.mt.ensure((size_t)nt * sizeof(vec3i) + 16));
    CKS(c->wr.mp.ensure((size_t)np * sizeof(vec3d) + 16));
    if (nt) CK(cudaMemcpyAsync(c->wr.mt.p, tris, (size_t)nt * sizeof(vec3i), cudaMemcpyHostToDevice, c->stream));
    if (np) CK(cudaMemcpyAsync(c->wr.mp.p, pts, (size_t)np * sizeof(vec3d), cudaMemcpyHostToDevice, c->stream));
    *dt = c->wr.mt.as<vec3i>();
    *dp = c->wr.mp.as<vec3d>();
    return N2M_OK;
}

n2m_status to_malloc(n2m_context *c, const unsigned char *d, size_t len, unsigned char **out, size_t *out_len) {
    unsigned char *h = (unsigned char *)malloc(std::max<size_t>(len, 1));
    if (!h) {
        n2m_set_error("host allocation failed");
        return N2M_ERR_OOM;
    }
    if (len && (cudaMemcpyAsync(h, d, len, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
                cudaStreamSynchronize(c->stream) != cudaSuccess)) {
        free(h);
        n2m_set_error("encoded mesh readback: %s", cudaGetErrorString(cudaGetLastError()));
        return N2M_ERR_CUDA;
    }
    *out = h;
    *out_len = len;
    return N2M_OK;
}

// encoded bytes -> file, through the context's pinned staging buffer in pieces (copy of piece k+1 overlaps the
// write of piece k)
n2m_status write_file(n2m_context *c, const char *fnm, const unsigned char *d, size_t len) {
    constexpr size_t PIECE = 32u << 20;
    const size_t cap = std::min(len, 2 * PIECE);
    if (c->wr.host_cap < cap) {
        if (c->wr.host) cudaFreeHost(c->wr.host);
        c->wr.host = nullptr;
        c->wr.host_cap = 0;
        CK(cudaHostAlloc(&c->wr.host, std::max<size_t>(cap, 1), cudaHostAllocDefault));
        c->wr.host_cap = cap;
    }
    FILE *f = fopen(fnm, "wb");
    if (!f) {
        n2m_set_error("cannot open %s for writing", fnm);
        return N2M_ERR_BAD_ARGS;
    }
    unsigned char *h = (unsigned char *)c->wr.host;
    n2m_status st = N2M_OK;
    size_t done = 0;
    int k = 0;
    // piece k goes to half (k & 1) of the staging buffer
    if (len && cudaMemcpyAsync(h, d, std::min(len, PIECE), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) st = N2M_ERR_CUDA;
    while (st == N2M_OK && done < len) {
        const size_t n = std::min(len - done, PIECE);
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
            st = N2M_ERR_CUDA;
            break;
        }
        const size_t next = done + n;
        if (next < len &&
            cudaMemcpyAsync(h + ((k + 1) & 1) * PIECE, d + next, std::min(len - next, PIECE), cudaMemcpyDeviceToHost,
                            c->stream) != cudaSuccess) {
            st = N2M_ERR_CUDA;
            break;
        }
        if (fwrite(h + (k & 1) * PIECE, 1, n, f) != n) {
            n2m_set_error("write to %s failed", fnm);
            st = N2M_ERR_BAD_ARGS;
            break;
        }
        done = next;
        k++;
    }
    cudaStreamSynchronize(c->stream);
    if (fclose(f) != 0 && st == N2M_OK) {
        n2m_set_error("write to %s failed", fnm);
        st = N2M_ERR_BAD_ARGS;
    }
    if (st == N2M_ERR_CUDA) n2m_set_error("mesh file readback: %s", cudaGetErrorString(cudaGetLastError()));
    return st;
}

n2m_status save_device(n2m_context *c, const char *fnm, const vec3i *dt, const vec3d *dp, int nt, int np, int gz) {
    if (!fnm) return N2M_ERR_BAD_ARGS;
    int fmt = mesh_format_of(fnm);
    std::string name(fnm);
    if (fmt < 0) {   // save_mesh appends ".mz3" to names it does not recognise
        name += ".mz3";
        fmt = N2M_FMT_MZ3;
    }
    const unsigned char *d;
    size_t len;
    CKS(encode_mesh_device(fmt, dt, dp, nt, np, gz != 0, c->wr, c->scan, c->stream, &d, &len));
    return write_file(c, name.c_str(), d, len);
}
}  // namespace

extern "C" n2m_status n2m_encode_mesh_device(n2m_context *c, int format, const vec3i *d_tris, const vec3d *d_pts,
                                             int ntri, int npt, int is_gz, unsigned char **out, size_t *out_len) {
    if (!c || !out || !out_len) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    const unsigned char *d;
    size_t len;
    CKS(encode_mesh_device(format, d_tris, d_pts, ntri, npt, is_gz != 0, c->wr, c->scan, c->stream, &d, &len));
    return to_malloc(c, d, len, out, out_len);
}

extern "C" n2m_status n2m_encode_mesh_to_device(n2m_context *c, int format, const vec3i *d_tris, const vec3d *d_pts,
                                                int ntri, int npt, int is_gz, const unsigned char **d_out,
                                                size_t *out_len) {
    if (!c || !d_out || !out_len) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    CKS(encode_mesh_device(format, d_tris, d_pts, ntri, npt, is_gz != 0, c->wr, c->scan, c->stream, d_out, out_len));
    CK(cudaStreamSynchronize(c->stream));
    return N2M_OK;
}

extern "C" n2m_status n2m_encode_mesh(n2m_context *c, int format, const vec3i *tris, const vec3d *pts, int ntri,
                                      int npt, int is_gz, unsigned char **out, size_t *out_len) {
    if (!c || !out || !out_len) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    const vec3i *dt;
    const vec3d *dp;
    CKS(upload_mesh(c, tris, pts, ntri, npt, &dt, &dp));
    const unsigned char *d;
    size_t len;
    CKS(encode_mesh_device(format, dt, dp, ntri, npt, is_gz != 0, c->wr, c->scan, c->stream, &d, &len));
    return to_malloc(c, d, len, out, out_len);
}

extern "C" n2m_status n2m_save_mesh_device(n2m_context *c, const char *fnm, const vec3i *d_tris, const vec3d *d_pts,
                                           int ntri, int npt, int is_gz) {
    if (!c) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    return save_device(c, fnm, d_tris, d_pts, ntri, npt, is_gz);
}

extern "C" n2m_status n2m_save_mesh(n2m_context *c, const char *fnm, const vec3i *tris, const vec3d *pts, int ntri,
                                    int npt, int is_gz) {
    if (!c) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    const vec3i *dt;
    const vec3d *dp;
    CKS(upload_mesh(c, tris, pts, ntri, npt, &dt, &dp));
    return save_device(c, fnm, dt, dp, ntri, npt, is_gz);
}

extern "C" int save_mesh(const char *fnm, vec3i *tris, vec3d *pts, int ntri, int npt, bool isGz) {
    n2m_context *c;
    n2m_status s = default_ctx(&c);
    if (s == N2M_OK) s = n2m_save_mesh(c, fnm, tris, pts, ntri, npt, isGz ? 1 : 0);
    if (s != N2M_OK) {
        report_failure("save_mesh", s);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

extern "C" n2m_status n2m_deflate_device(n2m_context *c, const void *d_src, size_t nbytes, int container,
                                         unsigned char **out, size_t *out_len) {
    if (!c || !out || !out_len || (nbytes && !d_src)) return N2M_ERR_BAD_ARGS;
    CK(cudaSetDevice(c->device));
    // the deflate kernels read whole aligned words up to 8 bytes past the end: work on a padded copy
    CKS(c->wr.pack.ensure(nbytes + 16));
    if (nbytes) CK(cudaMemcpyAsync(c->wr.pack.p, d_src, nbytes, cudaMemcpyDeviceToDevice, c->stream));
    CK(cudaMemsetAsync(c->wr.pack.as<unsigned char>() + nbytes, 0, 16, c->stream));
    size_t len;
    CKS(deflate_device(c->wr.pack.p, nbytes, container, c->wr.df, c->scan, c->stream, &len));
    CKS(deflate_check(c->wr.df, c->stream));
    return to_malloc(c, c->wr.df.out.as<unsigned char>(), len, out, out_len);
}

