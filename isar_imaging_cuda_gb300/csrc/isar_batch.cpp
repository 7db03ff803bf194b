// Batched imaging of many frames of uneven size in one CUDA graph, and the
// autotuner that picks launch parameters per frame shape and the number of
// concurrent lanes per batch.  No counterpart in the reference, which images
// one frame per isarMainSingle call (isar_imaging_export.cpp:208-212).
//
// Execution model.  Frames are grouped by shape (the full isar_radar).  Each
// shape owns up to `lanes` imaging contexts, each with its own stream; the
// frames of a shape are dealt round-robin to its lanes.  One batch run is
// captured once: the batch stream forks to every lane stream (event wait),
// each lane images its frames back to back (the per-frame chain of
// isar_image_device, recorded eagerly while capturing), and every lane joins
// the batch stream again.  The instantiated graph is cached per frame list
// and replayed with one cudaGraphLaunch.  Lanes use the cluster autofocus
// engine: one cooperative grid per frame would need all of its CTAs
// co-resident, which concurrent lanes cannot promise.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/isar_gb300.h"
#include "isar_kernels.h"

namespace {

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return isar::record_error(code, buf);
}

#define CU(call)                                                                                        \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return fail(ISAR_ECUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
#define TRY(x)                          \
    do {                                \
        const int rc_ = (x);            \
        if (rc_ != ISAR_OK) return rc_; \
    } while (0)

bool same_radar(const isar_radar& a, const isar_radar& b)
{
    return a.echo_num == b.echo_num && a.range_num == b.range_num && a.band_width == b.band_width && a.fc == b.fc &&
           a.Tp == b.Tp && a.Fs == b.Fs && a.data_type == b.data_type;
}

struct Lane {
    isar_ctx* ctx = nullptr;
    cudaStream_t st = nullptr;
    cudaEvent_t done = nullptr;
};

struct Shape {
    isar_radar r{};
    isar_tuning tuning{};
    bool tuned = false;
    std::vector<Lane> lanes;
};

struct BatchGraph {
    std::vector<isar_batch_frame> frames;
    int lanes = 0;
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;
    unsigned long long tick = 0;
};

bool same_frames(const std::vector<isar_batch_frame>& a, const isar_batch_frame* b, int n)
{
    if ((int)a.size() != n) return false;
    for (int i = 0; i < n; ++i)
        if (!same_radar(a[i].radar, b[i].radar) || a[i].d_echo != b[i].d_echo || a[i].d_velocity != b[i].d_velocity ||
            a[i].flags != b[i].flags || a[i].d_img != b[i].d_img)
            return false;
    return true;
}

}  // namespace

struct isar_batch {
    int dev = 0;
    cudaStream_t st = nullptr;
    bool own_stream = false;
    cudaEvent_t fork = nullptr;
    int lanes = 4;                 // lanes per shape (isar_batch_autotune picks it)
    const isar_wsnet* ws = nullptr;   // learned warm start of every lane, or null
    std::vector<std::unique_ptr<Shape>> shapes;
    std::vector<BatchGraph> graphs;
    unsigned long long tick = 0;
};

namespace {

void destroy_lane(Lane& l)
{
    if (l.done) cudaEventDestroy(l.done);
    if (l.ctx) isar_destroy(l.ctx);
    l = Lane{};
}

void drop_graphs(isar_batch* b)
{
    for (auto& g : b->graphs) cudaGraphExecDestroy(g.exec);
    b->graphs.clear();
}

Shape* shape_for(isar_batch* b, const isar_radar& r)
{
    for (auto& s : b->shapes)
        if (same_radar(s->r, r)) return s.get();
    return nullptr;
}

// The defaults of a new shape: the reference's parameters with the cluster
// autofocus engine (largest launchable cluster, 16 preferred).
int default_tuning(isar_ctx* c, isar_tuning* t)
{
    TRY(isar_get_tuning(c, t));
    if (t->af_cluster_max < 4) return fail(ISAR_ECUDA, "thread-block clusters of 4 CTAs cannot be launched here");
    t->af_cluster = t->af_cluster_max >= 16 ? 16 : t->af_cluster_max;
    return ISAR_OK;
}

// Instantiated batch graphs kept per batch (least recently used dropped):
// enough for a caller that rotates several buffer sets through the same
// frames (e.g. copy-in / compute / copy-out pipelines) next to a resident set.
constexpr size_t kBatchGraphs = 12;

int ensure_lanes(isar_batch* b, Shape* s, int n)
{
    while ((int)s->lanes.size() < n) {
        Lane l;
        int rc = isar_create(&l.ctx, &s->r, b->dev, nullptr);
        if (rc != ISAR_OK) return rc;
        l.st = static_cast<cudaStream_t>(isar_stream(l.ctx));
        if (cudaEventCreateWithFlags(&l.done, cudaEventDisableTiming) != cudaSuccess) {
            destroy_lane(l);
            return fail(ISAR_ECUDA, "cudaEventCreate failed");
        }
        if (!s->tuned) {
            rc = default_tuning(l.ctx, &s->tuning);
            if (rc != ISAR_OK) {
                destroy_lane(l);
                return rc;
            }
            s->tuned = true;
        }
        rc = isar_set_tuning(l.ctx, &s->tuning);
        if (rc == ISAR_OK && b->ws) rc = isar_set_warmstart(l.ctx, b->ws);
        if (rc != ISAR_OK) {
            destroy_lane(l);
            return rc;
        }
        s->lanes.push_back(l);
    }
    return ISAR_OK;
}

int check_frames(const isar_batch_frame* f, int n)
{
    if (!f || n <= 0) return fail(ISAR_EINVAL, "empty batch");
    for (int i = 0; i < n; ++i)
        if (!f[i].d_echo || !f[i].d_img) return fail(ISAR_EINVAL, "frame %d: null echo or image", i);
        else if (reinterpret_cast<uintptr_t>(f[i].d_echo) & 15)
            return fail(ISAR_EINVAL, "frame %d: echo buffer must be 16-byte aligned", i);
    return ISAR_OK;
}

// Records the whole batch on the batch stream (capturing or not).
int record_batch(isar_batch* b, const isar_batch_frame* f, int n, int lanes)
{
    // group by shape, deal frames round-robin to the shape's lanes
    std::vector<std::pair<Shape*, std::vector<std::vector<int>>>> plan;
    for (int i = 0; i < n; ++i) {
        Shape* s = shape_for(b, f[i].radar);
        if (!s) {
            b->shapes.emplace_back(new Shape());
            s = b->shapes.back().get();
            s->r = f[i].radar;
        }
        auto it = std::find_if(plan.begin(), plan.end(), [&](const auto& p) { return p.first == s; });
        if (it == plan.end()) {
            plan.emplace_back(s, std::vector<std::vector<int>>(lanes));
            it = plan.end() - 1;
        }
        auto& q = it->second;
        size_t k = 0;
        for (size_t j = 1; j < q.size(); ++j)
            if (q[j].size() < q[k].size()) k = j;
        q[k].push_back(i);
    }
    for (auto& p : plan) {
        int used = 0;
        for (auto& q : p.second) used += q.empty() ? 0 : 1;
        TRY(ensure_lanes(b, p.first, used));
    }
    CU(cudaEventRecord(b->fork, b->st));
    for (auto& p : plan) {
        int li = 0;
        for (auto& q : p.second) {
            if (q.empty()) continue;
            Lane& l = p.first->lanes[li++];
            CU(cudaStreamWaitEvent(l.st, b->fork, 0));
            for (int i : q) TRY(isar_image_device(l.ctx, f[i].d_echo, f[i].d_velocity, f[i].flags, f[i].d_img));
            CU(cudaEventRecord(l.done, l.st));
            CU(cudaStreamWaitEvent(b->st, l.done, 0));
        }
    }
    return ISAR_OK;
}

int capture_batch(isar_batch* b, const isar_batch_frame* f, int n, int lanes, BatchGraph* out)
{
    const long long n0 = isar_launch_count();
    CU(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeRelaxed));
    int rc = record_batch(b, f, n, lanes);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->st, &graph);
    if (rc != ISAR_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return fail(ISAR_ECUDA, "batch capture: %s", cudaGetErrorString(e));
    out->frames.assign(f, f + n);
    out->lanes = lanes;
    out->kernels = isar_launch_count() - n0;
    e = cudaGraphInstantiate(&out->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(ISAR_ECUDA, "batch graph instantiate: %s", cudaGetErrorString(e));
    return ISAR_OK;
}

// Median-free minimum of `reps` timed replays of `exec` on the batch stream, ms.
int time_graph(isar_batch* b, cudaGraphExec_t exec, int reps, float* ms)
{
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best = 1e30f;
    int rc = ISAR_OK;
    for (int r = 0; r < reps + 1 && rc == ISAR_OK; ++r) {
        if (cudaEventRecord(e0, b->st) != cudaSuccess || cudaGraphLaunch(exec, b->st) != cudaSuccess ||
            cudaEventRecord(e1, b->st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            rc = fail(ISAR_ECUDA, "timed batch replay failed: %s", cudaGetErrorString(cudaGetLastError()));
            break;
        }
        float t = 0.0f;
        cudaEventElapsedTime(&t, e0, e1);
        if (r > 0) best = std::min(best, t);   // first replay warms up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = best;
    return rc;
}

}  // namespace

// ---------------------------------------------------------------------------
// single-context autotuner
// ---------------------------------------------------------------------------
ISAR_API int isar_autotune(isar_ctx* c, const float* d_echo, const double* d_velocity, int flags, int engines,
                           isar_tuning* out)
{
    if (!c || !d_echo || !out) return fail(ISAR_EINVAL, "null argument");
    if ((engines & 3) == 0) return fail(ISAR_EINVAL, "engines must allow the cooperative (1) or cluster (2) engine");
    isar_tuning base;
    TRY(isar_get_tuning(c, &base));
    cudaStream_t st = static_cast<cudaStream_t>(isar_stream(c));
    // scratch image of the largest frame (echo_num <= 1024); tuning is a
    // set-up step, not the imaging path
    float* d_img = nullptr;
    CU(cudaMalloc(&d_img, (size_t)1024 * 512 * sizeof(float)));
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    auto timed = [&](const isar_tuning& t, float* ms) -> int {
        TRY(isar_set_tuning(c, &t));
        float best = 1e30f;
        for (int r = 0; r < 4; ++r) {
            CU(cudaEventRecord(e0, st));
            TRY(isar_image_device(c, d_echo, d_velocity, flags, d_img));
            CU(cudaEventRecord(e1, st));
            CU(cudaEventSynchronize(e1));
            float x = 0.0f;
            cudaEventElapsedTime(&x, e0, e1);
            if (r > 0) best = std::min(best, x);
        }
        TRY(isar_synchronize(c));
        *ms = best;
        return ISAR_OK;
    };
    isar_tuning best = base;
    std::vector<int> cls;
    if (engines & 1) cls.push_back(0);
    if (engines & 2)
        for (int cl : {16, 8, 4})
            if (cl <= base.af_cluster_max) cls.push_back(cl);
    if (cls.empty()) {
        cudaFree(d_img);
        return fail(ISAR_EINVAL, "no allowed autofocus engine can be launched here");
    }
    if (!(engines & 1) && best.af_cluster == 0) best.af_cluster = cls[0];
    if ((engines & 1) && !(engines & 2)) best.af_cluster = 0;
    best.af_tol = best.af_cluster ? base.af_tol : 0.0f;
    float best_ms = 0.0f;
    int rc = timed(best, &best_ms);
    // coordinate descent over the range-alignment knobs (the envelope path,
    // then the carried-envelope path's pair threshold and rows per CTA, then
    // the final transform's rows per CTA), then the engine
    const int em[] = {0, 1};
    const int pm[] = {1, 8, 32, 128, 512};
    const int rp[] = {1, 2, 4, 8, 16};
    const int rf[] = {1, 2, 4, 8};
    for (int pass = 0; pass < 5 && rc == ISAR_OK; ++pass) {
        if ((pass == 1 || pass == 2) && best.ra_rows_each_level == 0) continue;   // no effect on the spectral path
        const int* vals = pass == 0 ? em : pass == 1 ? pm : pass == 2 ? rp : pass == 3 ? rf : cls.data();
        const int nv = pass == 0 ? 2 : pass == 1 ? 5 : pass == 2 ? 5 : pass == 3 ? 4 : (int)cls.size();
        for (int i = 0; i < nv && rc == ISAR_OK; ++i) {
            isar_tuning t = best;
            int* knob = pass == 0   ? &t.ra_rows_each_level
                        : pass == 1 ? &t.ra_pair_min
                        : pass == 2 ? &t.ra_rows_per_cta
                        : pass == 3 ? &t.ra_rows_final
                                    : &t.af_cluster;
            if (*knob == vals[i]) continue;
            *knob = vals[i];
            if (pass == 4) t.af_tol = t.af_cluster ? base.af_tol : 0.0f;
            float ms = 0.0f;
            rc = timed(t, &ms);
            if (rc == ISAR_OK && ms < best_ms) {
                best_ms = ms;
                best = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_img);
    if (rc != ISAR_OK) {
        isar_set_tuning(c, &base);
        return rc;
    }
    TRY(isar_set_tuning(c, &best));
    TRY(isar_get_tuning(c, out));
    return ISAR_OK;
}

// ---------------------------------------------------------------------------
// batches
// ---------------------------------------------------------------------------
ISAR_API int isar_batch_create(isar_batch** out, int device, void* stream, int lanes)
{
    if (!out) return fail(ISAR_EINVAL, "null output");
    if (lanes < 0 || lanes > 128) return fail(ISAR_EINVAL, "lanes must be in [0, 128]");
    std::unique_ptr<isar_batch> b(new isar_batch());
    b->dev = device;
    CU(cudaSetDevice(device));
    if (stream) {
        b->st = static_cast<cudaStream_t>(stream);
    } else {
        CU(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
        b->own_stream = true;
    }
    CU(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    if (lanes > 0) b->lanes = lanes;
    *out = b.release();
    return ISAR_OK;
}

ISAR_API int isar_batch_destroy(isar_batch* b)
{
    if (!b) return ISAR_OK;
    cudaSetDevice(b->dev);
    cudaStreamSynchronize(b->st);
    drop_graphs(b);
    for (auto& s : b->shapes)
        for (auto& l : s->lanes) destroy_lane(l);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->own_stream) cudaStreamDestroy(b->st);
    delete b;
    return ISAR_OK;
}

ISAR_API void* isar_batch_stream(isar_batch* b) { return b ? b->st : nullptr; }

ISAR_API int isar_batch_run(isar_batch* b, const isar_batch_frame* f, int n)
{
    if (!b) return fail(ISAR_EINVAL, "null batch");
    TRY(check_frames(f, n));
    CU(cudaSetDevice(b->dev));
    ++b->tick;
    for (auto& g : b->graphs)
        if (g.lanes == b->lanes && same_frames(g.frames, f, n)) {
            g.tick = b->tick;
            CU(cudaGraphLaunch(g.exec, b->st));
            isar::launch_counter() += g.kernels;
            return ISAR_OK;
        }
    BatchGraph g;
    TRY(capture_batch(b, f, n, b->lanes, &g));
    g.tick = b->tick;
    if (b->graphs.size() >= kBatchGraphs) {
        auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                    [](const BatchGraph& x, const BatchGraph& y) { return x.tick < y.tick; });
        cudaGraphExecDestroy(lru->exec);
        b->graphs.erase(lru);
    }
    b->graphs.push_back(g);
    CU(cudaGraphLaunch(g.exec, b->st));
    isar::launch_counter() += g.kernels;
    return ISAR_OK;
}

ISAR_API int isar_batch_synchronize(isar_batch* b)
{
    if (!b) return fail(ISAR_EINVAL, "null batch");
    CU(cudaStreamSynchronize(b->st));
    for (auto& s : b->shapes)
        for (auto& l : s->lanes) TRY(isar_synchronize(l.ctx));
    return ISAR_OK;
}

ISAR_API int isar_batch_set_tuning(isar_batch* b, const isar_radar* shape, const isar_tuning* t)
{
    if (!b || !shape || !t) return fail(ISAR_EINVAL, "null argument");
    if (t->af_cluster == 0) return fail(ISAR_EINVAL, "batch lanes need the cluster autofocus engine");
    Shape* s = shape_for(b, *shape);
    if (!s) {
        b->shapes.emplace_back(new Shape());
        s = b->shapes.back().get();
        s->r = *shape;
    }
    TRY(ensure_lanes(b, s, 1));
    for (auto& l : s->lanes) TRY(isar_set_tuning(l.ctx, t));
    TRY(isar_get_tuning(s->lanes[0].ctx, &s->tuning));
    s->tuned = true;
    drop_graphs(b);
    return ISAR_OK;
}

ISAR_API int isar_batch_get_tuning(isar_batch* b, const isar_radar* shape, isar_tuning* out)
{
    if (!b || !shape || !out) return fail(ISAR_EINVAL, "null argument");
    Shape* s = shape_for(b, *shape);
    if (!s || !s->tuned) return fail(ISAR_ESTATE, "shape not seen by this batch");
    *out = s->tuning;
    return ISAR_OK;
}

ISAR_API int isar_batch_lanes(isar_batch* b) { return b ? b->lanes : 0; }

ISAR_API int isar_batch_set_warmstart(isar_batch* b, const isar_wsnet* net)
{
    if (!b) return fail(ISAR_EINVAL, "null batch");
    CU(cudaStreamSynchronize(b->st));
    for (auto& s : b->shapes)
        for (auto& l : s->lanes) TRY(isar_set_warmstart(l.ctx, net));
    b->ws = net;
    drop_graphs(b);
    return ISAR_OK;
}

/*
 * Autotunes `f`: per shape, the launch parameters on the first frame of that
 * shape (isar_autotune with the cluster engine only), then the lanes per
 * shape from {1, 2, 4, ..., 128} (up to the largest frame count of a shape)
 * jointly with the cluster size (16, 8 or 4 CTAs) by timing whole-batch graph
 * replays, then on the whole batch again the range-alignment envelope path
 * and rows per CTA (accumulate kernel, then final transform): with many
 * frames in flight fewer, longer CTAs beat the single-frame choice.  The next
 * isar_batch_run captures the chosen configuration.
 */
ISAR_API int isar_batch_autotune(isar_batch* b, const isar_batch_frame* f, int n, float* best_ms)
{
    if (!b) return fail(ISAR_EINVAL, "null batch");
    TRY(check_frames(f, n));
    CU(cudaSetDevice(b->dev));
    CU(cudaStreamSynchronize(b->st));
    drop_graphs(b);
    int most = 0;
    for (int i = 0; i < n; ++i) {
        Shape* s = shape_for(b, f[i].radar);
        if (!s) {
            b->shapes.emplace_back(new Shape());
            s = b->shapes.back().get();
            s->r = f[i].radar;
        }
        int cnt = 0;
        for (int k = 0; k < n; ++k) cnt += same_radar(f[k].radar, s->r) ? 1 : 0;
        most = std::max(most, cnt);
        if (s->lanes.empty() || !s->tuned) TRY(ensure_lanes(b, s, 1));
    }
    for (auto& sp : b->shapes) {
        Shape* s = sp.get();
        int first = -1;
        for (int i = 0; i < n && first < 0; ++i)
            if (same_radar(f[i].radar, s->r)) first = i;
        if (first < 0) continue;
        isar_tuning t{};
        TRY(isar_autotune(s->lanes[0].ctx, f[first].d_echo, f[first].d_velocity, f[first].flags, 2, &t));
        s->tuning = t;
        for (auto& l : s->lanes) TRY(isar_set_tuning(l.ctx, &t));
    }
    // applies fn to every shape's tuning (and its lanes)
    auto apply = [&](auto fn) -> int {
        for (auto& sp : b->shapes) {
            Shape* s = sp.get();
            fn(s->tuning);
            for (auto& l : s->lanes) TRY(isar_set_tuning(l.ctx, &s->tuning));
        }
        return ISAR_OK;
    };
    // whole-batch time of the current tuning with L lanes
    auto time_with = [&](int L, float* ms) -> int {
        BatchGraph g;
        TRY(capture_batch(b, f, n, L, &g));
        const int rc = time_graph(b, g.exec, 3, ms);
        cudaGraphExecDestroy(g.exec);
        return rc;
    };
    // lanes x cluster size: single-frame latency favours large clusters,
    // concurrent lanes can favour smaller ones
    auto set_cluster = [](int cl) {
        return [cl](isar_tuning& t) {
            if (cl <= t.af_cluster_max) t.af_cluster = cl;
        };
    };
    float best = 1e30f;
    int best_l = b->lanes, best_cl = 0;
    for (int cl : {16, 8, 4}) {
        TRY(apply(set_cluster(cl)));
        for (int L : {1, 2, 4, 8, 16, 32, 64, 128}) {
            if (L > 1 && L / 2 >= most) break;
            float ms = 0.0f;
            TRY(time_with(L, &ms));
            if (ms < best) {
                best = ms;
                best_l = L;
                best_cl = cl;
            }
        }
    }
    TRY(apply(set_cluster(best_cl)));
    // range-alignment knobs at the chosen lanes (coordinate descent): the
    // envelope path, the accumulate kernel's rows per CTA (carried-envelope
    // path only), the final transform's rows per CTA
    for (int field = 0; field < 3; ++field) {
        auto ref = [field](isar_tuning& t) -> int& {
            return field == 0 ? t.ra_rows_each_level : field == 1 ? t.ra_rows_per_cta : t.ra_rows_final;
        };
        std::vector<int> vals = {4, 8, 16, 32};
        if (field == 0) vals = {0, 1};
        if (field == 1) {
            bool any = false;
            for (auto& sp : b->shapes) any = any || sp->tuning.ra_rows_each_level;
            if (!any) continue;
        }
        std::vector<int> orig;   // per shape, kept unless a uniform value wins
        for (auto& sp : b->shapes) orig.push_back(ref(sp->tuning));
        int keep = -1;
        for (int v : vals) {
            TRY(apply([&](isar_tuning& t) { ref(t) = v; }));
            float ms = 0.0f;
            TRY(time_with(best_l, &ms));
            if (ms < best) {
                best = ms;
                keep = v;
            }
        }
        size_t i = 0;
        TRY(apply([&](isar_tuning& t) {
            ref(t) = keep >= 0 ? keep : orig[i];
            ++i;
        }));
    }
    b->lanes = best_l;
    if (best_ms) *best_ms = best;
    return ISAR_OK;
}
