// cvm_api.cpp -- host orchestration and the C ABI of cvmatch_gpu.h.
//
// Every public entry point funnels into one of two device pipelines:
//   run_solo   Match / MatchMap / MatchGray / matchU8 / Matcher.Find
//              (impl.go:1126-1155, matcher.go:83-130)
//   run_fleet  Fleet.FindAll (fleet.go:176-332)
// Both queue kernels on a stream and allocate their per-call workspace
// from a stream-ordered memory pool, so nothing synchronises until the
// host-buffer wrappers read their results back.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <limits>
#include <mutex>
#include <string>
#include <vector>
#include <atomic>
#include <tuple>

#include "cvm_internal.h"
#include "cvm_plan.h"

namespace cvm {

static std::atomic<uint64_t> g_launches{0};
void count_launches(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static thread_local int t_pdl = 0;
void set_pdl(int on) { t_pdl = on; }
int pdl_on() { return t_pdl; }

static thread_local std::string t_err;
void set_error_message(const char *msg) { t_err = msg; }

namespace {

int fail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

#define CVM_CUDA(call)                                                                     \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(CVM_ERR_CUDA, "cvmatch_gpu: %s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CVM_TRY(expr)        \
    do {                     \
        int rc_ = (expr);    \
        if (rc_ != CVM_OK) return rc_; \
    } while (0)

// ------------------------------------------------------------ device

struct DeviceState {
    std::once_flag once;
    int status = CVM_OK;
    std::string msg;
    int device = 0;
    int pageable = 0;  // the device reads pageable host memory coherently (cudaDevAttrPageableMemoryAccess)
    cudaMemPool_t pool = nullptr;
    std::mutex triMu;
    std::map<int, float2 *> tri;  // log2 n -> device twiddle table
};

DeviceState &dev() {
    static DeviceState d;
    return d;
}

int ensure_device() {
    DeviceState &d = dev();
    std::call_once(d.once, [&d]() {
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0) {
            d.status = CVM_ERR_NO_DEVICE;
            d.msg = std::string("cvmatch_gpu: no CUDA device: ") + cudaGetErrorString(e);
            return;
        }
        cudaGetDevice(&d.device);
        cudaDeviceProp prop;
        cudaGetDeviceProperties(&prop, d.device);
        if (prop.major != 10 || prop.minor != 3) {
            d.status = CVM_ERR_NO_DEVICE;
            char b[160];
            snprintf(b, sizeof b, "cvmatch_gpu: built for sm_103a, device %d is sm_%d%d", d.device,
                     prop.major, prop.minor);
            d.msg = b;
            return;
        }
        cudaDeviceGetAttribute(&d.pageable, cudaDevAttrPageableMemoryAccess, d.device);
        cudaMemPoolProps props;
        memset(&props, 0, sizeof props);
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = d.device;
        e = cudaMemPoolCreate(&d.pool, &props);
        if (e != cudaSuccess) {
            d.status = CVM_ERR_CUDA;
            d.msg = std::string("cvmatch_gpu: cudaMemPoolCreate: ") + cudaGetErrorString(e);
            return;
        }
        uint64_t keep = UINT64_MAX;  // keep freed workspace cached for the next call
        cudaMemPoolSetAttribute(d.pool, cudaMemPoolAttrReleaseThreshold, &keep);
        // the tensor-core DFT's tables (24 KB), before any call can be
        // inside a stream capture
        e = tc_init();
        if (e != cudaSuccess) {
            d.status = CVM_ERR_CUDA;
            d.msg = std::string("cvmatch_gpu: tensor-core tables: ") + cudaGetErrorString(e);
            return;
        }
    });
    if (d.status != CVM_OK) return fail(d.status, "%s", d.msg.c_str());
    // The library's state (memory pool, twiddle tables, per-thread
    // streams, Matcher and Fleet caches) lives on the device that was
    // current at its first call; a call made with another device current
    // would hand that state to launches on the wrong device.
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != d.device)
        return fail(CVM_ERR_UNSUPPORTED,
                    "cvmatch_gpu: the library is bound to CUDA device %d (current at its first call); the calling "
                    "thread's current device is %d",
                    d.device, cur);
    return CVM_OK;
}

// Per-thread non-blocking stream for the host-buffer entry points.
cudaStream_t thread_stream() {
    thread_local cudaStream_t s = nullptr;
    if (!s) cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    return s;
}

// Two per-thread side streams: st carries the template spectrum, st2 the
// window statistics; fork is recorded on the caller's stream once the
// channel count exists, join/joinStats when each chain is done.  A
// host-buffer call also moves its frame in on st2 (frame marks the end),
// while the caller's stream takes the template and the small setup.
struct SideStream {
    cudaStream_t st = nullptr, st2 = nullptr;
    cudaStream_t stats = nullptr;  // the caller's priority: a one-shot match's frame rows or late statistics
    cudaEvent_t fork = nullptr, join = nullptr, joinStats = nullptr, frame = nullptr;
    cudaEvent_t hsumDone = nullptr;  // a late statistics chain's horizontal sums
    cudaEvent_t prep = nullptr;      // a one-shot match's k_prep done
    cudaEvent_t rows = nullptr;      // a one-shot match's frame row transform done (stats stream)
    // a fleet's overlapped waves: the inverse rows of wave k on waveRows
    // beside the statistics and columns of wave k + 1 on the caller's stream
    cudaStream_t waveRows = nullptr;
    cudaEvent_t colsDone = nullptr, rowsDone[2] = {nullptr, nullptr};
};

SideStream &side_stream() {
    thread_local SideStream s;
    if (!s.st) {
        // The side chains gate the caller's stream: above its priority,
        // their CTAs are placed first as SMs free up (at the caller's
        // priority a one-CTA launch there waits tens of microseconds behind
        // the transforms).
        int least = 0, greatest = 0;
        cudaDeviceGetStreamPriorityRange(&least, &greatest);
        cudaStreamCreateWithPriority(&s.st, cudaStreamNonBlocking, greatest);
        cudaStreamCreateWithPriority(&s.st2, cudaStreamNonBlocking, greatest < least ? greatest + 1 : greatest);
        cudaStreamCreateWithPriority(&s.stats, cudaStreamNonBlocking, least);
        cudaEventCreateWithFlags(&s.fork, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.join, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.joinStats, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.frame, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.hsumDone, cudaEventDisableTiming);
        cudaStreamCreateWithFlags(&s.waveRows, cudaStreamNonBlocking);
        cudaEventCreateWithFlags(&s.colsDone, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.rowsDone[0], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.rowsDone[1], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.prep, cudaEventDisableTiming);
        cudaEventCreateWithFlags(&s.rows, cudaEventDisableTiming);
    }
    return s;
}

const float2 *dev_tri(int n) {
    DeviceState &d = dev();
    std::lock_guard<std::mutex> lk(d.triMu);
    const int l = ilog2(n);
    auto it = d.tri.find(l);
    if (it != d.tri.end()) return it->second;
    std::vector<float> t = tri_twiddles(n);
    if (t.empty()) t.assign(2, 0.f);
    float2 *p = nullptr;
    if (cudaMalloc(&p, t.size() * sizeof(float)) != cudaSuccess) return nullptr;
    if (cudaMemcpy(p, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    d.tri[l] = p;
    return p;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Bump allocator over one pool allocation.
struct Arena {
    char *base = nullptr;
    size_t used = 0;
    template <typename T>
    T *take(size_t count) {
        T *p = reinterpret_cast<T *>(base + used);
        used += align_up(count * sizeof(T), 256);
        return p;
    }
    static size_t bytes(size_t count, size_t elem) { return align_up(count * elem, 256); }
};

struct PoolBuf {
    void *p = nullptr;
    cudaStream_t st = nullptr;
    // stream-ordered free behind the work already queued on s
    void release(cudaStream_t s) {
        if (p) cudaFreeAsync(p, s);
        p = nullptr;
    }
    ~PoolBuf() {
        if (p) cudaFreeAsync(p, st);
    }
};

int pool_alloc(PoolBuf &b, size_t bytes, cudaStream_t st) {
    b.st = st;
    CVM_CUDA(cudaMallocFromPoolAsync(&b.p, bytes ? bytes : 256, dev().pool, st));
    return CVM_OK;
}

// Largest transforms the shared-memory kernels take (inverse rows hold a
// dftW row plus its accumulators; the column pass one dftH strip).
constexpr int kMaxDftW = 8192;
constexpr int kMaxDftH = 16384;

// ------------------------------------------------------------- geometry

// A plan with its tile grid and plan classes (main / shrunk last band).
struct Geom {
    Plan p;
    int dh2 = 0;
    TileGeom g;
    int nclass = 1;
    FftClass fc[2];
};

int make_geom(int tw, int th, int rw, int rh, int shrinkTH, Geom &G, const Plan *forced = nullptr) {
    G.p = forced ? *forced : make_plan(tw, th, rw, rh);
    if (G.p.dftW > kMaxDftW || G.p.dftH > kMaxDftH)
        return fail(CVM_ERR_UNSUPPORTED, "cvmatch_gpu: tile transform %dx%d exceeds the supported %dx%d",
                    G.p.dftW, G.p.dftH, kMaxDftW, kMaxDftH);
    G.dh2 = shrink_dh(G.p, rh, shrinkTH);
    TileGeom &g = G.g;
    g.ntx = (rw + G.p.blockW - 1) / G.p.blockW;
    g.nty = (rh + G.p.blockH - 1) / G.p.blockH;
    g.blockW = G.p.blockW;
    g.blockH = G.p.blockH;
    g.rwT = rw;
    g.rhT = rh;
    g.twL = tw;
    g.thL = th;
    g.tileFirst = 0;
    const int hwp = (int)align_up(G.p.hw, 16);
    const float2 *triW = dev_tri(G.p.dftW);
    if (!triW) return fail(CVM_ERR_CUDA, "cvmatch_gpu: twiddle table allocation failed");
    const int ntiles = g.ntx * g.nty;
    G.nclass = G.dh2 > 0 ? 2 : 1;
    for (int c = 0; c < G.nclass; c++) {
        FftClass &f = G.fc[c];
        f.n = G.p.dftW;
        f.log2n = ilog2(G.p.dftW);
        f.hw = G.p.hw;
        f.hwp = hwp;
        f.dftH = c == 0 ? G.p.dftH : G.dh2;
        f.log2H = ilog2(f.dftH);
        f.triW = triW;
        f.triH = dev_tri(f.dftH);
        if (!f.triH) return fail(CVM_ERR_CUDA, "cvmatch_gpu: twiddle table allocation failed");
        if (G.nclass == 1) {
            f.tileFirst = 0;
            f.ntiles = ntiles;
        } else if (c == 0) {
            f.tileFirst = 0;
            f.ntiles = ntiles - g.ntx;
        } else {
            f.tileFirst = ntiles - g.ntx;
            f.ntiles = g.ntx;
        }
    }
    return CVM_OK;
}

// The fast and mixed forms run the length-specialised kernels only
// (transforms of 2^5 .. 2^12 points); a plan with a longer transform (a
// template over ~4000 pixels on a side) runs the exact form's kernels
// instead -- the reference's own arithmetic, bit for bit -- for that match
// or fleet bucket.
bool fast_sizes_ok(const Geom &G) {
    for (int c = 0; c < G.nclass; c++)
        if (G.fc[c].log2n < 5 || G.fc[c].log2n > 12 || G.fc[c].log2H < 5 || G.fc[c].log2H > 12) return false;
    return true;
}

int effective_form(int form, const Geom &G) { return form != CVM_FORM_EXACT && !fast_sizes_ok(G) ? CVM_FORM_EXACT : form; }

// Geometry that loads one template as a single tile (template spectra).
void template_geom(const Geom &G, int tw, int th, TileGeom &tg, FftClass &tf) {
    tg = TileGeom();
    tg.twL = tw;
    tg.thL = th;
    tf = G.fc[0];
    tf.tileFirst = 0;
    tf.ntiles = 1;
}

size_t spec_elems(const FftClass &f, int cnS) { return (size_t)f.ntiles * cnS * f.dftH * f.hwp; }
size_t tspec_elems(const FftClass &f, int cnS) { return (size_t)cnS * f.dftH * f.hwp; }

// Template spectra on plan G for cnS channels: forward rows, forward
// columns scaled by 1/(dftW*dftH) (impl.go:535-553), then the shrunk-band
// gather (impl.go:591-610).  cnDev limits the channels on the device.
// The template spectrum, scaled by 1/(dftW*dftH) (buildTSpecSet,
// impl.go:520-561).  tsum (the fast form): per-channel template sums; the
// spectrum is then that of the zero-mean template area*T - sum(T), built
// from exact integer samples when area*255 < 2^24 (else T - mean), and
// scaled back by 1/area, so the correlation it yields is the numerator
// sum(I*T) - sum(I)*sum(T)/area directly.
int build_tspec(const Geom &G, const uint8_t *d_tpl, long long tstride, int step, int tw, int th,
                int cnS, const int *cnDev, float2 *ts0, float2 *ts1, cudaStream_t st,
                const int64_t *tsum = nullptr, const unsigned long long *tsumDev = nullptr, int selfSums = 0) {
    TileGeom tg;
    FftClass tf;
    template_geom(G, tw, th, tg, tf);
    float mul = 1.0f, sub[4] = {0.f, 0.f, 0.f, 0.f};
    const double area = double(tw) * double(th);
    const bool exact = area * 255.0 < 16777216.0;
    if (tsum || tsumDev || selfSums) mul = exact ? float(area) : 1.0f;
    if (tsum)
        for (int k = 0; k < 4; k++) sub[k] = exact ? float(tsum[k]) : float(double(tsum[k]) / area);
    // sums on the device (one-shot calls): sub = tsum / (1 or area)
    CVM_CUDA(launch_fwd_rows(d_tpl, tstride, step, cnS, cnDev, tg, tf, ts0, cnS, st, 0, "k_fwd_rows_tpl", mul,
                             tsum ? sub : nullptr, tsumDev, exact ? 1.0f : float(area), selfSums));
    const float scale = float(1.0 / (double(G.p.dftW) * double(G.p.dftH) * double(mul)));
    MemberSet none;
    memset(&none, 0, sizeof none);
    CVM_CUDA(launch_cols(0, ts0, ts0, cnS, tg, tf, 0, cnS, cnDev, scale, none, 1, st, "k_cols_tpl"));
    if (G.nclass == 2) CVM_CUDA(launch_shrink_gather(ts0, G.p.dftH, ts1, G.dh2, tf.hwp, cnS, st));
    return CVM_OK;
}

// ---------------------------------------------------------- solo pipeline

// The arithmetic of one-shot matches and Matcher.Find (cvm_set_form).
std::atomic<int> g_soloForm{CVM_FORM_EXACT};
int solo_form() { return g_soloForm.load(std::memory_order_relaxed); }

struct TemplateCache;  // a Matcher's per-geometry state

struct SoloJob {
    const uint8_t *img;
    long long istride;
    int iw, ih, step;
    int mode;     // 0: cn fixed; 1: colour, cn 3/4 decided by the alpha planes
    int cnFixed;
    const uint8_t *tpl;  // device template pixels (one-shot) -- or nullptr with cache
    long long tstride;
    int tw, th;
    const Geom *G;                // cached geometry (Matcher) or nullptr
    const float2 *cachedTs[2];    // cached template spectra
    const DevParams *cachedP;     // cached template statistics
    float *map;
    cvm_result *out;
    int frameOnSide;  // the frame arrives on the second side stream (its frame event)
    int form;         // CVM_FORM_EXACT, _FAST or _MIXED (cached spectra must be of this form)
    const Plan *plan; // the tile plan (one-shot; nullptr: the tuned plan, or newGoPlan)
};

int run_solo(const SoloJob &J, cudaStream_t st);

// ------------------------------------------------------------ autotuner
//
// The fast and mixed forms may run any tile plan (the exact form keeps
// newGoPlan, impl.go:246-295: its bits depend on the plan).  The first
// fast-form call of a shape times up to four candidate plans
// (plan_candidates: newGoPlan's choice and the best of a GPU cost proxy)
// on the call's own inputs -- each run once to warm up, then twice from a
// cold L2 between CUDA events on the call's stream, the faster of the two
// counting -- and keeps the fastest if it beats
// newGoPlan's by more than 3 %; the choice is cached per (frame size,
// template size, channel mode, form) for the life of the process, so every
// later call of the shape (one-shot calls and Matchers alike) runs the same
// plan and gives the same results.  A call made while its stream is being
// captured into a graph runs newGoPlan's plan and tunes nothing.
struct TuneKey {
    int iw, ih, tw, th, mode, cn, step, form;
    bool operator<(const TuneKey &o) const {
        return std::tie(iw, ih, tw, th, mode, cn, step, form) <
               std::tie(o.iw, o.ih, o.tw, o.th, o.mode, o.cn, o.step, o.form);
    }
};
struct TuneEntry {
    Plan plan;
    int n = 0;
    Plan cand[4];
    float ms[4] = {0, 0, 0, 0};
};
std::mutex g_tuneMu;
std::map<TuneKey, TuneEntry> g_tune;
std::atomic<int> g_autotune{1};

// The plan a fast-form one-shot match of J's shape runs (tuning it first
// when needed); *out = newGoPlan's plan when tuning is off or not possible.
int solo_plan(const SoloJob &J, cudaStream_t st, Plan *out) {
    const int rw = J.iw - J.tw + 1, rh = J.ih - J.th + 1;
    *out = make_plan(J.tw, J.th, rw, rh);
    if (J.form == CVM_FORM_EXACT || !g_autotune.load()) return CVM_OK;
    const TuneKey key{J.iw, J.ih, J.tw, J.th, J.mode, J.mode == 1 ? 0 : J.cnFixed, J.step, J.form};
    {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            *out = it->second.plan;
            return CVM_OK;
        }
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return CVM_OK;
    }
    std::vector<Plan> cands = plan_candidates(J.tw, J.th, rw, rh, 4);
    TuneEntry ent;
    ent.plan = *out;
    if (cands.size() > 1) {
        thread_local cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (!e0) {
            CVM_CUDA(cudaEventCreate(&e0));
            CVM_CUDA(cudaEventCreate(&e1));
        }
        // Each timed run starts from a cold L2 (a transient buffer twice the
        // L2's size cleared before it), as a frame that just arrived does.
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev().device);
        void *flush = nullptr;
        const size_t flushBytes = (size_t)2 * (l2 > 0 ? l2 : (64 << 20));
        if (cudaMalloc(&flush, flushBytes) != cudaSuccess) {
            cudaGetLastError();
            flush = nullptr;
        }
        int best = 0;
        int rc = CVM_OK;
        for (size_t i = 0; i < cands.size() && rc == CVM_OK; i++) {
            SoloJob T = J;
            T.plan = &cands[i];
            rc = run_solo(T, st);  // warm-up (workspace, twiddle tables)
            float msBest = 0;
            for (int r = 0; r < 2 && rc == CVM_OK; r++) {
                if (flush) cudaMemsetAsync(flush, 0, flushBytes, st);
                cudaEventRecord(e0, st);
                rc = run_solo(T, st);
                cudaEventRecord(e1, st);
                if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(CVM_ERR_CUDA, "cvmatch_gpu: autotune timing failed");
                float ms = 0;
                cudaEventElapsedTime(&ms, e0, e1);
                if (r == 0 || ms < msBest) msBest = ms;
            }
            ent.cand[ent.n] = cands[i];
            ent.ms[ent.n] = msBest;
            ent.n++;
            if (msBest < ent.ms[best]) best = (int)i;
        }
        if (flush) cudaFree(flush);
        if (rc != CVM_OK) return rc;
        // cands[0] is newGoPlan's choice whenever it qualifies
        const bool baseFirst = cands[0].dftW == out->dftW && cands[0].dftH == out->dftH;
        if (!baseFirst || ent.ms[best] < 0.97f * ent.ms[0]) ent.plan = cands[best];
    }
    std::lock_guard<std::mutex> lk(g_tuneMu);
    auto ins = g_tune.emplace(key, ent);  // another thread may have tuned the shape meanwhile
    *out = ins.first->second.plan;
    return CVM_OK;
}

int run_solo(const SoloJob &J, cudaStream_t st) {
    const int rw = J.iw - J.tw + 1, rh = J.ih - J.th + 1;
    Geom local;
    const Geom *G = J.G;
    if (!G) {
        Plan p;
        if (J.plan)
            p = *J.plan;
        else
            CVM_TRY(solo_plan(J, st, &p));
        CVM_TRY(make_geom(J.tw, J.th, rw, rh, J.th, local, &p));
        G = &local;
    }
    const int cnS = J.mode == 1 ? 4 : J.cnFixed;
    const SepGrid sg = sep_grid(rw, rh);
    int nparts = 0, partOff[2] = {0, 0};
    for (int c = 0; c < G->nclass; c++) {
        int P = 0;
        partOff[c] = nparts;
        nparts += G->fc[c].ntiles * inv_rows_ctas_per_tile(G->fc[c], G->g.blockH, &P);
    }
    const size_t hElems = (size_t)stat_pitch(cnS) * J.ih * sg.hp;
    // a tall template with a fixed channel count: 16-row block sums of the
    // window sums, from which every vertical band starts
    // (the block sums are u32: 16 rows of the squared window sum, 16 * tw *
    // cn * 255^2, must stay below 2^32)
    const size_t bElems = (J.mode == 0 && J.th >= 64 && 16ull * J.tw * J.cnFixed * 65025ull < (1ull << 32))
                              ? (size_t)stat_pitch(J.cnFixed) * (J.ih / 16) * sg.hp
                              : 0;
    size_t bytes = Arena::bytes(1, sizeof(DevParams)) + Arena::bytes(1, sizeof(DevFrame)) +
                   Arena::bytes(nparts, sizeof(Partial)) + Arena::bytes(hElems, sizeof(unsigned int)) +
                   Arena::bytes((size_t)rw * rh, sizeof(float2)) + (bElems ? Arena::bytes(bElems, sizeof(unsigned int)) : 0);
    // (a Matcher's cached spectra were built for the same effective form)
    const int form = effective_form(J.form, *G);
    const bool fast = form != CVM_FORM_EXACT;
    // one channel: the fused forward + conj-multiply + inverse column pass
    // already yields the single correlation spectrum the fast form sums to
    const bool fastSum = fast && !(J.mode == 0 && J.cnFixed == 1);
    for (int c = 0; c < G->nclass; c++) {
        bytes += Arena::bytes(spec_elems(G->fc[c], cnS), sizeof(float2));
        if (fastSum) bytes += Arena::bytes(spec_elems(G->fc[c], 1), sizeof(float2));
        if (!J.cachedP) bytes += Arena::bytes(tspec_elems(G->fc[c], cnS), sizeof(float2));
    }
    PoolBuf buf;
    CVM_TRY(pool_alloc(buf, bytes, st));
    Arena A;
    A.base = static_cast<char *>(buf.p);
    DevParams *P = A.take<DevParams>(1);
    DevFrame *F = A.take<DevFrame>(1);
    Partial *parts = A.take<Partial>(nparts);
    unsigned int *H = A.take<unsigned int>(hElems);
    unsigned int *blk = bElems ? A.take<unsigned int>(bElems) : nullptr;
    float2 *lanes = A.take<float2>((size_t)rw * rh);
    float2 *spec[2] = {nullptr, nullptr}, *sum[2] = {nullptr, nullptr};
    const float2 *ts[2] = {J.cachedTs[0], J.cachedTs[1]};
    float2 *tsOwn[2] = {nullptr, nullptr};
    for (int c = 0; c < G->nclass; c++) {
        spec[c] = A.take<float2>(spec_elems(G->fc[c], cnS));
        if (fastSum) sum[c] = A.take<float2>(spec_elems(G->fc[c], 1));
        if (!J.cachedP) {
            tsOwn[c] = A.take<float2>(tspec_elems(G->fc[c], cnS));
            ts[c] = tsOwn[c];
        }
    }
    CVM_CUDA(cudaMemsetAsync(F, 0, sizeof(DevFrame), st));
    if (J.cachedP)
        CVM_CUDA(cudaMemcpyAsync(P, J.cachedP, sizeof(DevParams), cudaMemcpyDeviceToDevice, st));
    else
        CVM_CUDA(cudaMemsetAsync(P, 0, sizeof(DevParams), st));
    MemberSet ms;
    memset(&ms, 0, sizeof ms);
    ms.solo.tspec[0] = ts[0];
    ms.solo.tspec[1] = ts[1];
    ms.solo.pIdx = 0;
    ms.solo.tw = J.tw;
    ms.solo.th = J.th;
    ms.solo.rw = rw;
    ms.solo.rh = rh;
    ms.solo.partBase = 0;
    ms.solo.outIdx = 0;
    ms.solo.roiX0 = 0;
    ms.solo.roiY0 = 0;
    ms.solo.roiX1 = rw;
    ms.solo.roiY1 = rh;
    ms.params = P;
    ms.map = J.map;
    ms.lanes = lanes;
    ms.lanesStride = 0;
    ms.form = form;
    // One short launch (k_prep: the template statistics, the parent's
    // alpha scan, the channel count) on st, then chains: the frame's row
    // transform (on st, or on the rows stream beside k_prep); the template
    // spectrum on the first side stream; the window statistics on the
    // second; the column and inverse-row passes on st.  A launch that does
    // not start first does not get SMs back from one that did (priority
    // orders only the CTAs waiting for a slot), so k_prep is the launch
    // that is ready first.
    SideStream &ss = side_stream();
    // A one-shot colour match on a device-resident frame starts its template
    // spectrum at once, beside k_prep: all four channels (the frame's alpha
    // plane decides later whether the fourth is used) and, in the fast form,
    // the zero-mean samples from sums the row kernel takes itself -- the
    // spectrum depends on nothing k_prep computes.  (With a host frame in
    // flight the same early chain measured slower end to end, with the
    // ingest kernel and with the copy engine alike: host-buffer calls keep
    // the template behind the frame.)
    const bool early = !J.frameOnSide && !J.cachedP && J.mode == 1 && (long long)J.tw * J.th <= 65536;
    if (early) {
        CVM_CUDA(cudaEventRecord(ss.fork, st));  // the template and the pool's spectrum buffers
        CVM_CUDA(cudaStreamWaitEvent(ss.st, ss.fork, 0));
        CVM_TRY(build_tspec(*G, J.tpl, J.tstride, J.step, J.tw, J.th, cnS, nullptr, tsOwn[0], tsOwn[1], ss.st,
                            nullptr, nullptr, fast ? 1 : 0));
        CVM_CUDA(cudaEventRecord(ss.join, ss.st));
    }
    // A fast-form colour match with a short template (the fused column pass
    // dominates; the statistics have slack until the inverse rows) queues its
    // horizontal sums behind the frame's row transform, at the caller's
    // priority, so they fill the SMs the transforms leave instead of
    // displacing the row transform; otherwise the statistics start after
    // k_prep, above it.
    const bool statsLate = fastSum && J.th <= 64;
    // Otherwise, on a frame of 2^20 pixels or more, the frame's row
    // transform of every channel the alpha scans cannot drop (all but a
    // colour match's alpha plane) runs on the rows stream (the caller's
    // priority) from before k_prep, which only the alpha plane's transform,
    // the statistics and the template chain wait for; k_prep, ready at once
    // on the caller's stream, still places its CTAs first.  (A small frame
    // or a late statistics chain loses more to the extra cross-stream
    // waits and the side chains it exposes: a 640x480 gray match with a
    // 64x48 template 70.3 -> 73.4 us, a 1920x1080 colour match with a 96x32
    // template 92.8 -> 96.6 us in the fast form; the same match in the exact
    // form 118.5 -> 113 us, a 3840x2160 gray match with a 256x256 template
    // 209.6 -> 202.7 us in the fast form.)
    const bool split = !statsLate && (long long)J.iw * J.ih >= (1LL << 20);
    if (J.frameOnSide) CVM_CUDA(cudaStreamWaitEvent(st, ss.frame, 0));
    if (split) {
        CVM_CUDA(cudaEventRecord(ss.fork, st));  // the frame, P and F zeroed, the pool's buffers
        CVM_CUDA(cudaStreamWaitEvent(ss.stats, ss.fork, 0));
    }
    CVM_CUDA(launch_prep(J.cachedP ? nullptr : J.tpl, J.tstride, J.tw, J.th, J.step, cnS,
                         J.mode == 1 ? J.img : nullptr, J.istride, J.iw, J.ih, P, 1, J.cachedP ? 0 : 1, J.mode,
                         J.cnFixed, F, st));
    // the fast form transforms the frame offset by -128 (zero-mean templates)
    const float off[4] = {128.f, 128.f, 128.f, 128.f};
    if (split) {
        for (int c = 0; c < G->nclass; c++)
            CVM_CUDA(launch_fwd_rows(J.img, J.istride, J.step, J.mode == 1 ? 3 : cnS, nullptr, G->g, G->fc[c],
                                     spec[c], cnS, ss.stats, 0, nullptr, 1.0f, fast ? off : nullptr));
        CVM_CUDA(cudaEventRecord(ss.rows, ss.stats));
    }
    cudaStream_t sst = statsLate ? ss.stats : ss.st2;
    CVM_CUDA(cudaEventRecord(ss.prep, st));
    if (!early) CVM_CUDA(cudaStreamWaitEvent(ss.st, ss.prep, 0));
    CVM_CUDA(cudaStreamWaitEvent(sst, ss.prep, 0));
    if (!statsLate) {
        CVM_CUDA(launch_sep_stats(J.img, J.istride, J.step, J.iw, J.ih, ms, 1, J.tw, rw, sg,
                                  J.mode == 1 ? 3 : J.cnFixed, J.mode == 1 ? 4 : J.cnFixed, H, 0, sst, 0, nullptr,
                                  nullptr, blk));
        CVM_CUDA(cudaEventRecord(ss.joinStats, sst));
    }
    if (!J.cachedP && !early)
        CVM_TRY(build_tspec(*G, J.tpl, J.tstride, J.step, J.tw, J.th, cnS, &P->cn, tsOwn[0], tsOwn[1], ss.st,
                            nullptr, fast ? P->tsum : nullptr));
    if (!early) CVM_CUDA(cudaEventRecord(ss.join, ss.st));
    if (split) {
        // a colour match's alpha plane, when the alpha scans chose four channels
        if (J.mode == 1)
            for (int c = 0; c < G->nclass; c++)
                CVM_CUDA(launch_fwd_rows(J.img, J.istride, J.step, 4, &P->cn, G->g, G->fc[c], spec[c], cnS, st, 3,
                                         nullptr, 1.0f, fast ? off : nullptr));
    } else {
        // every channel the device chose, one launch; with late statistics
        // it places its CTAs while k_prep finishes (programmatic dependent
        // launch)
        PdlScope pdl(statsLate);
        for (int c = 0; c < G->nclass; c++)
            CVM_CUDA(launch_fwd_rows(J.img, J.istride, J.step, cnS, &P->cn, G->g, G->fc[c], spec[c], cnS, st, 0,
                                     nullptr, 1.0f, fast ? off : nullptr));
    }
    if (statsLate) {
        // the horizontal sums at the caller's priority, the vertical pass
        // (which gates the inverse rows) back above it on the second side stream
        CVM_CUDA(launch_sep_stats(J.img, J.istride, J.step, J.iw, J.ih, ms, 1, J.tw, rw, sg,
                                  J.mode == 1 ? 3 : J.cnFixed, J.mode == 1 ? 4 : J.cnFixed, H, 0, sst, 0, ss.st2,
                                  ss.hsumDone, blk));
        CVM_CUDA(cudaEventRecord(ss.joinStats, ss.st2));
    }
    if (split) CVM_CUDA(cudaStreamWaitEvent(st, ss.rows, 0));
    // Several channels, fast form: transforms up to 512 tall run every
    // channel of a column strip in one CTA (mode 4: forward, channel sum of
    // the conj-products, one inverse); taller ones store the forward
    // column spectra of every channel (in place) and sum them in a second
    // pass (mode 3).
    int colMode[2] = {1, 1};
    for (int c = 0; c < G->nclass; c++)
        if (fastSum) colMode[c] = G->fc[c].log2H <= 9 ? 4 : 3;
    // With late statistics (their chain has slack, the template chain too)
    // each transform launch follows a transform kernel on st and places its
    // CTAs while that one finishes; the event waits on the side chains stay
    // whole dependencies.  (A 1920x1080 colour match with a 96x32 template:
    // 92.6 -> 90.7 us; on a 640x480 gray match with a 64x48 template, whose
    // template chain gates the column pass, the frame transform's earlier
    // CTAs cost that chain SMs: 68.4 -> 72.9 us, so the others launch
    // plainly.)
    PdlScope pdl(statsLate);
    for (int c = 0; c < G->nclass; c++)
        if (colMode[c] == 3) {
            MemberSet none;
            memset(&none, 0, sizeof none);
            CVM_CUDA(launch_cols(0, spec[c], spec[c], cnS, G->g, G->fc[c], c, cnS, &P->cn, 1.0f, none, 1, st));
        }
    CVM_CUDA(cudaStreamWaitEvent(st, ss.join, 0));
    for (int c = 0; c < G->nclass; c++) {
        const FftClass &f = G->fc[c];
        ms.scratch[c] = fastSum ? sum[c] : spec[c];
        ms.scratchStride[c] = 0;
        CVM_CUDA(launch_cols(colMode[c], spec[c], spec[c], cnS, G->g, f, c, cnS, nullptr, 1.0f, ms, 1, st));
    }
    CVM_CUDA(cudaStreamWaitEvent(st, ss.joinStats, 0));
    for (int c = 0; c < G->nclass; c++)
        CVM_CUDA(launch_inv_rows(G->g, G->fc[c], c, fast ? 1 : cnS, ms, 1, G->g.blockH, partOff[c], nparts, parts,
                                 &F->normDone, J.out, st));
    return CVM_OK;
}

// ---------------------------------------------------------- validation

int check_match_args(int iw, int ih, long long istride, long long tstride, int tw, int th, int cn,
                     int step) {
    if (cn < 1 || cn > 4 || step < cn || tw < 1 || th < 1 || tw > iw || th > ih ||
        istride < (long long)iw * step || tstride < (long long)tw * step)
        return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d, cn=%d step=%d)", tw, th,
                    iw, ih, cn, step);
    if ((int64_t)tw * th > stats_cap(cn))
        return fail(CVM_ERR_STATS_CAP,
                    "cvmatch: template area %dx%d exceeds the exact-statistics bound for cn=%d", tw, th, cn);
    return CVM_OK;
}

// alphaConst on the host (cvmatch.go:146-168).  Only the validation of
// Match needs it on the host: its error text and its statistics cap depend
// on the channel count the alpha planes select (cvmatch.go:82-86).
bool host_alpha_const(const uint8_t *pix, long long stride, int w, int h) {
    const uint8_t a = pix[3];
    for (int y = 0; y < h; y++) {
        const uint8_t *row = pix + (long long)y * stride;
        for (int x = 0; x < w; x++)
            if (row[4 * x + 3] != a) return false;
    }
    return true;
}

// matchU8's argument checks for Match's RGBA inputs.  The device decides
// the channel count; the host repeats the alpha scan only when the check
// itself depends on it (a failing size check, or an area above the cn=4
// statistics cap).
int check_match_rgba(const uint8_t *parent, long long pstride, int pw, int ph, const uint8_t *sub,
                     long long sstride, int sw, int sh) {
    const bool sizesOk = sw <= pw && sh <= ph && pstride >= (long long)pw * 4 && sstride >= (long long)sw * 4;
    if (sizesOk && (int64_t)sw * sh <= stats_cap(4)) return CVM_OK;
    int cn = 4;
    if (pstride >= (long long)pw * 4 && sstride >= (long long)sw * 4 && host_alpha_const(parent, pstride, pw, ph) &&
        host_alpha_const(sub, sstride, sw, sh))
        cn = 3;
    return check_match_args(pw, ph, pstride, sstride, sw, sh, cn, 4);
}

int check_image(const void *p, int w, int h) {
    if (!p) return fail(CVM_ERR_NIL_IMAGE, "cvmatch: nil image");
    if (w <= 0 || h <= 0) return fail(CVM_ERR_EMPTY_IMAGE, "cvmatch: empty image");
    return CVM_OK;
}

// Copies a host image to a device buffer with a 128-byte aligned pitch.
// Per-thread page-locked staging for small pageable inputs (templates,
// small frames): the copy out of it is asynchronous, so a call's launches
// are queued while its frame is still in flight -- a pageable copy holds
// the host until the stream reaches it.  Each slot's last copy is fenced
// by an event that the next use waits for (normally long complete: the
// host-buffer entry points synchronise before returning).
struct Staging {
    void *p = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
    ~Staging() {
        if (p) cudaFreeHost(p);
        if (done) cudaEventDestroy(done);
    }
};

Staging *staging(size_t n, int slot) {
    thread_local Staging b[2];
    Staging &s = b[slot & 1];
    if (!s.done && cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    cudaEventSynchronize(s.done);
    if (s.cap < n) {
        if (s.p) cudaFreeHost(s.p);
        s.p = nullptr;
        s.cap = 0;
        const size_t cap = align_up(n, size_t(1) << 16);
        if (cudaHostAlloc(&s.p, cap, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        s.cap = cap;
    }
    return &s;
}

int upload_image(PoolBuf &b, const uint8_t *src, long long stride, int w, int h, int bpp,
                 long long *pitch, cudaStream_t st, int stageSlot = 0) {
    const size_t row = (size_t)w * bpp;
    *pitch = (long long)align_up(row, 128);
    CVM_TRY(pool_alloc(b, (size_t)*pitch * h, st));
    // Page-locked caller memory that the device can address is read by a
    // kernel over the host link (several times the copy engine's rate for
    // a frame); anything else goes through the copy engine.
    cudaPointerAttributes at;
    if ((size_t)row * h >= (size_t(1) << 20) && cudaPointerGetAttributes(&at, src) == cudaSuccess &&
        at.type == cudaMemoryTypeHost && at.devicePointer) {
        CVM_CUDA(launch_ingest(b.p, (size_t)*pitch, at.devicePointer, (size_t)stride, row, h, st));
        return CVM_OK;
    }
    cudaGetLastError();  // an unregistered pointer's query leaves no error behind
    // A device that reads pageable host memory coherently (a Grace host's
    // NVLink-C2C address translation) takes the caller's ordinary memory the
    // same way: no synchronous staged copy by the driver, so the transfer
    // overlaps the call's queued launches as a page-locked frame's does.
    // The caller's buffer stays valid until the call returns (it
    // synchronises before returning).
    if (dev().pageable && (size_t)row * h >= (size_t(64) << 10)) {
        CVM_CUDA(launch_ingest(b.p, (size_t)*pitch, src, (size_t)stride, row, h, st));
        return CVM_OK;
    }
    if (row * h <= (size_t(4) << 20)) {
        Staging *sg = staging(row * h, stageSlot);
        if (sg) {
            unsigned char *stg = static_cast<unsigned char *>(sg->p);
            for (int y = 0; y < h; y++) memcpy(stg + (size_t)y * row, src + (size_t)y * stride, row);
            CVM_CUDA(cudaMemcpy2DAsync(b.p, (size_t)*pitch, stg, row, row, h, cudaMemcpyHostToDevice, st));
            CVM_CUDA(cudaEventRecord(sg->done, st));
            return CVM_OK;
        }
    }
    CVM_CUDA(cudaMemcpy2DAsync(b.p, (size_t)*pitch, src, (size_t)stride, row, h, cudaMemcpyHostToDevice, st));
    return CVM_OK;
}

// One-shot host-buffer match: upload both images, run, read back.
// Occurrence extraction requested from a one-shot call: the map stays on
// the device and only the occurrences come back.
struct PeakReq {
    float thresh;
    int rx, ry;
    int32_t *xy;
    int maxPeaks;
    int32_t *count;
};

// A per-thread page-locked result slot the device writes through its
// mapped address: the one-shot calls read their extrema from it after the
// stream synchronises, with no device-to-host copy behind the last launch.
cvm_result *host_result_slot(cvm_result **dev) {
    struct Slot {
        cvm_result *h = nullptr, *d = nullptr;
        ~Slot() {
            if (h) cudaFreeHost(h);
        }
    };
    thread_local Slot s;
    if (!s.h) {
        void *h = nullptr, *d = nullptr;
        if (cudaHostAlloc(&h, sizeof(cvm_result), cudaHostAllocMapped) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        if (cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess || !d) {
            cudaGetLastError();
            cudaFreeHost(h);
            return nullptr;
        }
        s.h = static_cast<cvm_result *>(h);
        s.d = static_cast<cvm_result *>(d);
    }
    *dev = s.d;
    return s.h;
}

int host_solo(const uint8_t *img, long long istride, int iw, int ih, const uint8_t *tpl, long long tstride,
              int tw, int th, int mode, int cnFixed, int step, int grayFromRgba, float *map,
              cvm_result *out, const PeakReq *pk = nullptr) {
    CVM_TRY(ensure_device());
    cudaStream_t st = thread_stream();
    SideStream &ss = side_stream();
    PoolBuf bi, bt, gi, gt, bm, bo;
    long long ip, tp;
    const int bpp = grayFromRgba ? 4 : step;
    // The frame moves in on the second side stream (the long transfer,
    // started first); the template and the setup of the launches proceed on
    // the caller's stream meanwhile, which waits for the frame only where it
    // first reads it.  The side stream's statistics chain is ordered after
    // that wait by the fork event.
    CVM_TRY(upload_image(bi, img, istride, iw, ih, bpp, &ip, ss.st2, 0));
    CVM_CUDA(cudaEventRecord(ss.frame, ss.st2));
    CVM_TRY(upload_image(bt, tpl, tstride, tw, th, bpp, &tp, st, 1));
    const uint8_t *dImg = static_cast<const uint8_t *>(bi.p), *dTpl = static_cast<const uint8_t *>(bt.p);
    if (grayFromRgba) {
        CVM_CUDA(cudaStreamWaitEvent(st, ss.frame, 0));
        long long gp = (long long)align_up((size_t)iw, 128), gtp = (long long)align_up((size_t)tw, 128);
        CVM_TRY(pool_alloc(gi, (size_t)gp * ih, st));
        CVM_TRY(pool_alloc(gt, (size_t)gtp * th, st));
        CVM_CUDA(launch_gray(dImg, ip, iw, ih, static_cast<uint8_t *>(gi.p), gp, st));
        CVM_CUDA(launch_gray(dTpl, tp, tw, th, static_cast<uint8_t *>(gt.p), gtp, st));
        dImg = static_cast<const uint8_t *>(gi.p);
        dTpl = static_cast<const uint8_t *>(gt.p);
        ip = gp;
        tp = gtp;
    }
    const int rw = iw - tw + 1, rh = ih - th + 1;
    float *dMap = nullptr;
    if (map || pk) {
        CVM_TRY(pool_alloc(bm, (size_t)rw * rh * sizeof(float), st));
        dMap = static_cast<float *>(bm.p);
    }
    cvm_result *dOut = nullptr, *hOut = host_result_slot(&dOut);
    if (!hOut) {
        CVM_TRY(pool_alloc(bo, sizeof(cvm_result), st));
        dOut = static_cast<cvm_result *>(bo.p);
    }
    SoloJob J;
    memset(&J, 0, sizeof J);
    J.form = solo_form();
    J.img = dImg;
    J.istride = ip;
    J.iw = iw;
    J.ih = ih;
    J.step = step;
    J.mode = mode;
    J.cnFixed = cnFixed;
    J.tpl = dTpl;
    J.tstride = tp;
    J.tw = tw;
    J.th = th;
    J.map = dMap;
    J.out = dOut;
    J.frameOnSide = !grayFromRgba;
    CVM_TRY(run_solo(J, st));
    if (map) CVM_CUDA(cudaMemcpyAsync(map, dMap, (size_t)rw * rh * sizeof(float), cudaMemcpyDeviceToHost, st));
    PoolBuf bp;
    if (pk) {
        const size_t nsc = peaks_scratch_ints(rw, rh);
        const size_t xyBytes = (size_t)std::max(pk->maxPeaks, 0) * 2 * sizeof(int32_t);
        CVM_TRY(pool_alloc(bp, (nsc + 1) * sizeof(int) + xyBytes, st));
        int *scr = static_cast<int *>(bp.p), *dCount = scr + nsc;
        int32_t *dXY = reinterpret_cast<int32_t *>(dCount + 1);
        CVM_CUDA(launch_peaks(dMap, rw, rh, pk->thresh, pk->rx, pk->ry, scr, dXY, pk->maxPeaks, dCount, st));
        CVM_CUDA(cudaMemcpyAsync(pk->count, dCount, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
        if (xyBytes) CVM_CUDA(cudaMemcpyAsync(pk->xy, dXY, xyBytes, cudaMemcpyDeviceToHost, st));
    }
    if (!hOut) CVM_CUDA(cudaMemcpyAsync(out, bo.p, sizeof(cvm_result), cudaMemcpyDeviceToHost, st));
    // the device buffers go back to the pool in stream order now, so the
    // host's frees overlap the device work instead of following the wait
    bi.release(st);
    bt.release(st);
    gi.release(st);
    gt.release(st);
    bm.release(st);
    bp.release(st);
    bo.release(st);
    CVM_CUDA(cudaStreamSynchronize(st));
    if (hOut) *out = *hOut;
    return CVM_OK;
}

const cvm_result kFlatResult = {1.f, 0, 0, 1.f, 0, 0};

}  // namespace
}  // namespace cvm

using namespace cvm;

// ================================================================ Matcher

struct MatcherGeom {
    int rw = 0, rh = 0;
    int form = CVM_FORM_EXACT;  // the arithmetic the spectra were built for
    Geom G;
    float2 *ts[2] = {nullptr, nullptr};
    ~MatcherGeom() {
        for (auto p : ts)
            if (p) cudaFree(p);
    }
};

struct cvm_matcher {
    int w = 0, h = 0, step = 0;
    bool aConst = false;
    int64_t tsum[4] = {0, 0, 0, 0};
    int64_t varSum = 0;
    uint8_t *dPix = nullptr;    // compact device copy, stride w*step
    DevParams *dP = nullptr;    // template statistics (raw sums), computed once
    std::mutex mu;
    std::shared_ptr<MatcherGeom> geom;
    ~cvm_matcher() {
        if (dPix) cudaFree(dPix);
        if (dP) cudaFree(dP);
    }
};

namespace {

// The Matcher's cached plan and spectra for one result size, built once
// under the handle's lock (the double-checked cache of matcher.go:114-126).
int matcher_geom(cvm_matcher *m, const uint8_t *dParent, long long pstride, int pw, int ph, int form, cudaStream_t st,
                 cvm_result *dOut, std::shared_ptr<MatcherGeom> &out) {
    const int rw = pw - m->w + 1, rh = ph - m->h + 1;
    std::lock_guard<std::mutex> lk(m->mu);
    if (m->geom && m->geom->rw == rw && m->geom->rh == rh && m->geom->form == form) {
        out = m->geom;
        return CVM_OK;
    }
    auto g = std::make_shared<MatcherGeom>();
    g->rw = rw;
    g->rh = rh;
    g->form = form;
    // the plan a one-shot match of this shape runs (tuned on this frame in
    // the fast forms), so Find and Match stay identical
    Plan plan;
    {
        SoloJob T;
        memset(&T, 0, sizeof T);
        T.form = form;
        T.img = dParent;
        T.istride = pstride;
        T.iw = pw;
        T.ih = ph;
        T.step = m->step;
        T.mode = m->step == 4 ? 1 : 0;
        T.cnFixed = m->step == 4 ? 4 : 1;
        T.tpl = m->dPix;
        T.tstride = (long long)m->w * m->step;
        T.tw = m->w;
        T.th = m->h;
        T.out = dOut;  // the tuning runs' results are overwritten by the call's own
        CVM_TRY(solo_plan(T, st, &plan));
    }
    CVM_TRY(make_geom(m->w, m->h, rw, rh, m->h, g->G, &plan));
    const int cnS = m->step;  // colour: all four channels (cn is decided per frame)
    for (int c = 0; c < g->G.nclass; c++)
        CVM_CUDA(cudaMalloc(&g->ts[c], tspec_elems(g->G.fc[c], cnS) * sizeof(float2)));
    cudaStream_t bst = thread_stream();
    CVM_TRY(build_tspec(g->G, m->dPix, (long long)m->w * m->step, m->step, m->w, m->h, cnS, nullptr, g->ts[0],
                        g->ts[1], bst, effective_form(form, g->G) != CVM_FORM_EXACT ? m->tsum : nullptr));
    CVM_CUDA(cudaStreamSynchronize(bst));
    m->geom = g;
    out = g;
    return CVM_OK;
}

int matcher_find_dev(cvm_matcher *m, const uint8_t *dParent, long long pstride, int pw, int ph,
                     cvm_result *dOut, cudaStream_t st) {
    if (m->w > pw || m->h > ph)
        return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d)", m->w, m->h, pw, ph);
    if (pstride < (long long)pw * m->step)
        return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d)", m->w, m->h, pw, ph);
    if (m->varSum == 0) {
        CVM_CUDA(upload_bytes(dOut, &kFlatResult, sizeof kFlatResult, st));
        return CVM_OK;
    }
    const int form = solo_form();
    std::shared_ptr<MatcherGeom> g;
    CVM_TRY(matcher_geom(m, dParent, pstride, pw, ph, form, st, dOut, g));
    SoloJob J;
    memset(&J, 0, sizeof J);
    J.form = form;
    J.img = dParent;
    J.istride = pstride;
    J.iw = pw;
    J.ih = ph;
    J.step = m->step;
    J.mode = m->step == 4 ? 1 : 0;
    J.cnFixed = 1;
    J.tw = m->w;
    J.th = m->h;
    J.G = &g->G;
    J.cachedTs[0] = g->ts[0];
    J.cachedTs[1] = g->ts[1];
    J.cachedP = m->dP;
    J.out = dOut;
    return run_solo(J, st);
}

}  // namespace

// ================================================================== Fleet

struct FleetBucketGeom {
    Geom G;
    int form = CVM_FORM_EXACT;    // the fleet's form, or exact where the plan exceeds the fast kernels
    SepGrid sg;
    int nparts = 0, partOff[2] = {0, 0};
    int rwMax = 0, rhMax = 0;
    int cnS = 1;
    std::vector<float2 *> ts;     // per member: class 0, class 1 (owned)
    DevMember *table = nullptr;   // bucket members in bucket order
    std::vector<DevMember> tabHost;  // its host copy
    uint64_t roiGen = 0;          // the fleet's ROI generation the table holds
    std::vector<int> members;
    size_t memberScratch[2] = {0, 0};
    ~FleetBucketGeom() {
        for (auto p : ts)
            if (p) cudaFree(p);
        if (table) cudaFree(table);
    }
};

struct FleetGeom {
    int pw = 0, ph = 0;
    int form = CVM_FORM_EXACT;  // the form the spectra were built for
    std::vector<std::unique_ptr<FleetBucketGeom>> bg;
};

struct cvm_fleet {
    std::vector<cvm_matcher *> ms;
    int step = 0;
    std::vector<Bucket> buckets;
    DevParams *dP = nullptr;  // per member template statistics
    std::mutex mu;
    std::shared_ptr<FleetGeom> geom;
    std::vector<int32_t> roi;  // per member x, y, w, h in frame pixels (w <= 0: the whole frame)
    uint64_t roiGen = 0;       // bumped by every cvm_fleet_set_roi
    int form = CVM_FORM_EXACT; // arithmetic of the member tails (cvm_fleet_set_form)
    int waveMembers = 0;       // members per wave of tails (0: by the 4 GB workspace budget)
    int statsMode = CVM_STATS_KERNEL;  // or CVM_STATS_EPILOGUE (cvm_fleet_set_stats)
    int overlapWaves = 1;      // cvm_fleet_set_overlap
    Plan forcedPlan;           // every bucket's plan when dftW > 0 (the autotuner's trial fleets)
    ~cvm_fleet() {
        if (dP) cudaFree(dP);
    }
};

namespace {

// Budget for one wave of member tails' column-pass output.
constexpr size_t kWaveBytes = size_t(4) << 30;

// Member i's region of interest as result positions [r0, r2) x [r1, r3)
// on a frame whose results span rw x rh: the positions whose tw x th
// window lies inside the ROI (all of them without an ROI; empty when the
// ROI cannot hold the template).  Returns false for "no ROI".
bool member_roi(const cvm_fleet *f, int i, int rw, int rh, int tw, int th, int r[4]) {
    r[0] = 0;
    r[1] = 0;
    r[2] = rw;
    r[3] = rh;
    if (f->roi.empty() || f->roi[4 * i + 2] <= 0 || f->roi[4 * i + 3] <= 0) return false;
    const int x = f->roi[4 * i], y = f->roi[4 * i + 1], w = f->roi[4 * i + 2], h = f->roi[4 * i + 3];
    r[0] = std::max(x, 0);
    r[1] = std::max(y, 0);
    r[2] = std::min(x + w - tw + 1, rw);
    r[3] = std::min(y + h - th + 1, rh);
    if (r[2] <= r[0] || r[3] <= r[1]) r[0] = r[1] = r[2] = r[3] = 0;  // empty
    return true;
}

void table_roi(const cvm_fleet *f, const FleetBucketGeom &bg, std::vector<DevMember> &tab) {
    for (size_t pos = 0; pos < bg.members.size(); pos++) {
        DevMember &d = tab[pos];
        int r[4];
        member_roi(f, bg.members[pos], d.rw, d.rh, d.tw, d.th, r);
        d.roiX0 = r[0];
        d.roiY0 = r[1];
        d.roiX1 = r[2];
        d.roiY1 = r[3];
    }
}

// Per parent size: every bucket's plan and every member's spectrum on its
// bucket's plan (buildGeom, fleet.go:337-390), plus the device member
// tables the tail kernels index.
int fleet_find_dev(cvm_fleet *f, const uint8_t *dParent, long long pstride, int pw, int ph, cvm_result *dOut,
                   cudaStream_t st);

// The fleet half of the autotuner: a bucket's plan in the fast forms.  The
// cost of a plan is measured on trial fleets of the bucket's own members
// (k and 2k of them, spread over the bucket) on the caller's frame, each
// run from a cold L2: the difference gives the per-member tail cost, the
// rest the frame's shared cost, and the bucket's cost is shared + n x
// per-member.  newGoPlan's plan (fleet.go:356-365) is kept unless another
// candidate beats it by more than 3 %.  Cached per (frame size, bucket
// maxima, members, step, form) for the process.
struct FleetTuneKey {
    int pw, ph, tw, th, step, form, n;
    bool operator<(const FleetTuneKey &o) const {
        return std::tie(pw, ph, tw, th, step, form, n) < std::tie(o.pw, o.ph, o.tw, o.th, o.step, o.form, o.n);
    }
};
struct FleetTuneEntry {
    Plan plan;
    int n = 0;
    static constexpr int kCands = 8;
    Plan cand[kCands];
    float perMember[kCands] = {}, shared[kCands] = {}, total[kCands] = {};
};
std::map<FleetTuneKey, FleetTuneEntry> g_fleetTune;

int tune_bucket_plan(cvm_fleet *f, const Bucket &b, const uint8_t *dParent, long long pstride, int pw, int ph,
                     cudaStream_t st, Plan *out) {
    const int rwF = pw - b.tw + 1, rhF = ph - b.th + 1;
    *out = make_plan(b.tw, b.th, rwF, rhF);
    const int nm = (int)b.members.size();
    if (f->form == CVM_FORM_EXACT || !g_autotune.load() || nm < 4 || !dParent) return CVM_OK;
    const FleetTuneKey key{pw, ph, b.tw, b.th, f->step, f->form, nm};
    {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        auto it = g_fleetTune.find(key);
        if (it != g_fleetTune.end()) {
            *out = it->second.plan;
            return CVM_OK;
        }
    }
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return CVM_OK;
    }
    std::vector<Plan> cands = plan_candidates(b.tw, b.th, rwF, rhF, FleetTuneEntry::kCands);
    FleetTuneEntry ent;
    ent.plan = *out;
    if (cands.size() > 1) {
        CVM_CUDA(cudaStreamSynchronize(st));  // the frame, written on the caller's stream
        cudaStream_t ts = thread_stream();
        thread_local cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (!e0) {
            CVM_CUDA(cudaEventCreate(&e0));
            CVM_CUDA(cudaEventCreate(&e1));
        }
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev().device);
        const size_t flushBytes = (size_t)2 * (l2 > 0 ? l2 : (64 << 20));
        void *flush = nullptr;
        if (cudaMalloc(&flush, flushBytes) != cudaSuccess) {
            cudaGetLastError();
            flush = nullptr;
        }
        const int k1 = std::max(2, std::min(8, nm / 2)), k2 = std::min(nm, 2 * k1);
        cvm_result *dOut = nullptr;
        if (cudaMalloc(&dOut, (size_t)k2 * sizeof(cvm_result)) != cudaSuccess) {
            cudaGetLastError();
            if (flush) cudaFree(flush);
            return CVM_OK;  // nothing to time with: newGoPlan's plan
        }
        int rc = CVM_OK, best = 0;
        for (size_t c = 0; c < cands.size() && rc == CVM_OK; c++) {
            float t[2] = {0, 0};
            for (int which = 0; which < 2 && rc == CVM_OK; which++) {
                const int k = which ? k2 : k1;
                cvm_fleet trial;
                trial.step = f->step;
                trial.form = f->form;
                trial.statsMode = f->statsMode;
                trial.forcedPlan = cands[c];
                Bucket one;
                one.tw = b.tw;
                one.th = b.th;
                for (int i = 0; i < k; i++) {
                    trial.ms.push_back(f->ms[b.members[(size_t)i * nm / k]]);
                    one.members.push_back(i);
                }
                trial.buckets.push_back(one);
                if (cudaMalloc(&trial.dP, (size_t)k * sizeof(DevParams)) != cudaSuccess) {
                    rc = fail(CVM_ERR_CUDA, "cvmatch_gpu: autotune workspace");
                    break;
                }
                for (int i = 0; i < k && rc == CVM_OK; i++)
                    if (cudaMemcpy(trial.dP + i, trial.ms[i]->dP, sizeof(DevParams), cudaMemcpyDeviceToDevice) !=
                        cudaSuccess)
                        rc = fail(CVM_ERR_CUDA, "cvmatch_gpu: autotune workspace");
                if (rc == CVM_OK) rc = fleet_find_dev(&trial, dParent, pstride, pw, ph, dOut, ts);  // geometry + warm-up
                float msBest = 0;
                for (int r = 0; r < 2 && rc == CVM_OK; r++) {
                    if (flush) cudaMemsetAsync(flush, 0, flushBytes, ts);
                    cudaEventRecord(e0, ts);
                    rc = fleet_find_dev(&trial, dParent, pstride, pw, ph, dOut, ts);
                    cudaEventRecord(e1, ts);
                    if (cudaEventSynchronize(e1) != cudaSuccess) rc = fail(CVM_ERR_CUDA, "cvmatch_gpu: autotune timing failed");
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (r == 0 || ms < msBest) msBest = ms;
                }
                if (rc == CVM_OK) cudaStreamSynchronize(ts);
                t[which] = msBest;
            }
            const float per = k2 > k1 ? std::max(0.f, (t[1] - t[0]) / (float)(k2 - k1)) : t[0] / (float)k1;
            const float shared = std::max(0.f, t[0] - per * (float)k1);
            ent.cand[ent.n] = cands[c];
            ent.perMember[ent.n] = per;
            ent.shared[ent.n] = shared;
            ent.total[ent.n] = shared + per * (float)nm;
            if (ent.total[ent.n] < ent.total[best]) best = ent.n;
            ent.n++;
        }
        cudaFree(dOut);
        if (flush) cudaFree(flush);
        if (rc != CVM_OK) return rc;
        const bool baseFirst = cands[0].dftW == out->dftW && cands[0].dftH == out->dftH;
        if (!baseFirst || ent.total[best] < 0.97f * ent.total[0]) ent.plan = cands[best];
    }
    std::lock_guard<std::mutex> lk(g_tuneMu);
    auto ins = g_fleetTune.emplace(key, ent);
    *out = ins.first->second.plan;
    return CVM_OK;
}

// The fast forms' buckets: the reference's (bucketize, fleet.go:111-171),
// each split in two where its shorter members would otherwise run tile rows
// they do not need (every member's tail runs every tile of its bucket's
// grid).  Costs in transform points (tiles x dftW x dftH of newGoPlan's
// plan for a part's maxima): a part's member tails cost points x members,
// its frame spectra about points x 3 (measured on C4: 6.4 us per frame tile
// against 2.2 us per member tile); a bucket is split at the member height
// that minimises the sum over both parts when that beats the whole bucket
// by more than 5 % and each part holds at least 32 members: the model
// leaves out each bucket's fixed costs (its launches, its waves' tails, the
// tuner's own plans), which smaller parts do not amortise (C4's 256
// members split 73 + 183, predicted -6.2 %, measured 9.28 -> 9.16 ms; the
// 1080p stream's 64 members split 29 + 35, predicted -3.5 %, measured
// 1.45 -> 1.61 ms per frame).  Members keep their construction order
// within each part.  The exact form keeps
// the reference's buckets (its bits follow from the bucket's plan).
std::vector<Bucket> fast_buckets(const cvm_fleet *f, int pw, int ph) {
    auto points = [&](int tw, int th) -> long long {
        const int rw = pw - tw + 1, rh = ph - th + 1;
        if (tw < 1 || th < 1 || rw < 1 || rh < 1) return 0;
        const Plan p = make_plan(tw, th, rw, rh);
        return (long long)((rw + p.blockW - 1) / p.blockW) * ((rh + p.blockH - 1) / p.blockH) * p.dftW * p.dftH;
    };
    std::vector<Bucket> out;
    for (const Bucket &b : f->buckets) {
        const long long n = (long long)b.members.size();
        const long long whole = points(b.tw, b.th) * (n + 3);
        std::vector<int> hs;
        for (int i : b.members) hs.push_back(f->ms[i]->h);
        std::sort(hs.begin(), hs.end());
        hs.erase(std::unique(hs.begin(), hs.end()), hs.end());
        long long best = whole;
        int bestT = -1;
        for (int T : hs) {
            if (T >= b.th) continue;
            int twA = 0, twB = 0, thB = 0;
            long long nA = 0, nB = 0;
            for (int i : b.members) {
                const cvm_matcher *m = f->ms[i];
                if (m->h <= T) {
                    twA = std::max(twA, m->w);
                    nA++;
                } else {
                    twB = std::max(twB, m->w);
                    thB = std::max(thB, m->h);
                    nB++;
                }
            }
            if (nA < 32 || nB < 32) continue;
            const long long c = points(twA, T) * (nA + 3) + points(twB, thB) * (nB + 3);
            if (c < best) {
                best = c;
                bestT = T;
            }
        }
        if (bestT < 0 || best * 100 > whole * 95) {
            out.push_back(b);
            continue;
        }
        Bucket lo, hi;
        for (int i : b.members) {
            const cvm_matcher *m = f->ms[i];
            Bucket &d = m->h <= bestT ? lo : hi;
            d.tw = std::max(d.tw, m->w);
            d.th = std::max(d.th, m->h);
            d.members.push_back(i);
        }
        // the taller part first: the last wave's inverse rows have nothing
        // left to overlap, and the shorter part's waves carry fewer tiles
        out.push_back(hi);
        out.push_back(lo);
    }
    return out;
}

int fleet_geom(cvm_fleet *f, const uint8_t *dParent, long long pstride, int pw, int ph, cudaStream_t cst,
               std::shared_ptr<FleetGeom> &out) {
    std::lock_guard<std::mutex> lk(f->mu);
    if (f->geom && f->geom->pw == pw && f->geom->ph == ph) {
        out = f->geom;
        return CVM_OK;
    }
    auto fg = std::make_shared<FleetGeom>();
    fg->pw = pw;
    fg->ph = ph;
    fg->form = f->form;
    cudaStream_t st = thread_stream();
    const std::vector<Bucket> buckets =
        f->form != CVM_FORM_EXACT && f->forcedPlan.dftW == 0 ? fast_buckets(f, pw, ph) : f->buckets;
    for (const Bucket &b : buckets) {
        auto bg = std::make_unique<FleetBucketGeom>();
        const int rwF = pw - b.tw + 1, rhF = ph - b.th + 1;
        Plan plan;
        if (f->forcedPlan.dftW > 0)
            plan = f->forcedPlan;
        else
            CVM_TRY(tune_bucket_plan(f, b, dParent, pstride, pw, ph, cst, &plan));
        CVM_TRY(make_geom(b.tw, b.th, rwF, rhF, b.th, bg->G, &plan));
        bg->form = effective_form(f->form, bg->G);
        const bool bfast = bg->form != CVM_FORM_EXACT;
        bg->cnS = f->step;
        bg->members = b.members;
        const Geom &G = bg->G;
        for (int mi : b.members) {
            bg->rwMax = std::max(bg->rwMax, pw - f->ms[mi]->w + 1);
            bg->rhMax = std::max(bg->rhMax, ph - f->ms[mi]->h + 1);
        }
        bg->sg = sep_grid(bg->rwMax, bg->rhMax);
        int nparts = 0;
        for (int c = 0; c < G.nclass; c++) {
            int P = 0;
            bg->partOff[c] = nparts;
            nparts += G.fc[c].ntiles * inv_rows_ctas_per_tile(G.fc[c], G.fc[c].dftH, &P, bfast,
                                                              bg->form == CVM_FORM_MIXED && G.fc[c].log2n == 10);
        }
        bg->nparts = nparts;
        std::vector<DevMember> tab(b.members.size());
        for (size_t pos = 0; pos < b.members.size(); pos++) {
            cvm_matcher *m = f->ms[b.members[pos]];
            float2 *t[2] = {nullptr, nullptr};
            for (int c = 0; c < G.nclass; c++) {
                CVM_CUDA(cudaMalloc(&t[c], tspec_elems(G.fc[c], bg->cnS) * sizeof(float2)));
                bg->ts.push_back(t[c]);
            }
            CVM_TRY(build_tspec(G, m->dPix, (long long)m->w * m->step, m->step, m->w, m->h, bg->cnS, nullptr,
                                t[0], t[1], st, bfast ? m->tsum : nullptr));
            DevMember &d = tab[pos];
            memset(&d, 0, sizeof d);
            d.tspec[0] = t[0];
            d.tspec[1] = t[1];
            d.pIdx = b.members[pos];
            d.tw = m->w;
            d.th = m->h;
            d.rw = pw - m->w + 1;
            d.rh = ph - m->h + 1;
            d.partBase = (int)pos * nparts;
            d.outIdx = b.members[pos];
        }
        table_roi(f, *bg, tab);
        bg->roiGen = f->roiGen;
        bg->tabHost = tab;
        CVM_CUDA(cudaMalloc(&bg->table, tab.size() * sizeof(DevMember)));
        CVM_CUDA(cudaMemcpy(bg->table, tab.data(), tab.size() * sizeof(DevMember), cudaMemcpyHostToDevice));
        // the fast form's member tails keep one channel-summed spectrum per tile
        for (int c = 0; c < G.nclass; c++)
            bg->memberScratch[c] = spec_elems(G.fc[c], bfast ? 1 : bg->cnS);
        fg->bg.push_back(std::move(bg));
    }
    CVM_CUDA(cudaStreamSynchronize(st));
    f->geom = fg;
    out = fg;
    return CVM_OK;
}

int fleet_find_dev(cvm_fleet *f, const uint8_t *dParent, long long pstride, int pw, int ph, cvm_result *dOut,
                   cudaStream_t st) {
    const int n = (int)f->ms.size();
    for (int i = 0; i < n; i++) {
        cvm_matcher *m = f->ms[i];
        if (m->w > pw || m->h > ph)
            return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d)", m->w, m->h, pw, ph);
    }
    if (pstride < (long long)pw * f->step)
        return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d)", f->ms[0]->w, f->ms[0]->h, pw, ph);
    for (int i = 0; i < n; i++)
        if (f->ms[i]->varSum == 0) {
            // a flat member scores 1 everywhere: its first result position
            // (impl.go:1137-1144), inside its region of interest if it has one
            cvm_matcher *m = f->ms[i];
            int r[4];
            cvm_result fr = kFlatResult;
            if (member_roi(f, i, pw - m->w + 1, ph - m->h + 1, m->w, m->h, r)) {
                if (r[2] > r[0]) {
                    fr.min_x = fr.max_x = r[0];
                    fr.min_y = fr.max_y = r[1];
                } else {
                    fr.min_v = fr.max_v = std::numeric_limits<float>::quiet_NaN();
                    fr.min_x = fr.min_y = fr.max_x = fr.max_y = -1;
                }
            }
            CVM_CUDA(upload_bytes(dOut + i, &fr, sizeof fr, st));
        }
    if (f->buckets.empty()) return CVM_OK;
    std::shared_ptr<FleetGeom> fg;
    CVM_TRY(fleet_geom(f, dParent, pstride, pw, ph, st, fg));
    {
        // regions of interest changed since the member tables were built
        std::lock_guard<std::mutex> lk(f->mu);
        for (auto &bgp : fg->bg) {
            FleetBucketGeom &bg = *bgp;
            if (bg.roiGen == f->roiGen) continue;
            table_roi(f, bg, bg.tabHost);
            CVM_CUDA(upload_bytes(bg.table, bg.tabHost.data(), bg.tabHost.size() * sizeof(DevMember), st));
            bg.roiGen = f->roiGen;
        }
    }
    const int cnS = f->step;
    size_t frameBytes = 0, partBytes = 0, waveBytes = 0;
    std::vector<int> wave(fg->bg.size());
    for (size_t b = 0; b < fg->bg.size(); b++) {
        const FleetBucketGeom &bg = *fg->bg[b];
        size_t fb = 0, per = 0;
        for (int c = 0; c < bg.G.nclass; c++) {
            fb += Arena::bytes(spec_elems(bg.G.fc[c], cnS), sizeof(float2));
            per += bg.memberScratch[c] * sizeof(float2);
        }
        const size_t lanesPer = (size_t)bg.rwMax * bg.rhMax;
        const int nparts = bg.nparts;
        per += lanesPer * sizeof(float2);
        frameBytes = std::max(frameBytes, fb);
        partBytes = std::max(partBytes, Arena::bytes((size_t)bg.members.size() * nparts, sizeof(Partial)));
        int w = (int)std::max<size_t>(1, kWaveBytes / std::max<size_t>(per, 1));
        if (f->waveMembers > 0) w = std::min(w, f->waveMembers);
        const int nmB = (int)bg.members.size();
        w = std::min<int>(w, nmB);
        // the budget's wave count with equal waves, not a short last one
        // (C4's 256 members: 4 x 64 instead of 78 + 78 + 78 + 22, 9.44 ->
        // 9.34 ms with the waves overlapped)
        if (f->waveMembers == 0 && w > 0) {
            const int nwv = (nmB + w - 1) / w;
            w = (nmB + nwv - 1) / nwv;
        }
        wave[b] = w;
        size_t wb = Arena::bytes((size_t)w * lanesPer, sizeof(float2));
        for (int c = 0; c < bg.G.nclass; c++) wb += Arena::bytes((size_t)w * bg.memberScratch[c], sizeof(float2));
        waveBytes = std::max(waveBytes, wb);
    }
    // one set of row prefixes for every member (each differences it at its own width)
    const int cnP = f->step == 4 ? 4 : 1;
    const int hpP = (int)align_up((size_t)pw + 1, 32);
    const size_t prefixElems = (size_t)(cnP == 4 ? 6 : stat_pitch(cnP)) * ph * hpP;
    // and their 16-row block sums (the main block), from which each band of
    // every member's vertical slide starts
    // (u32 sums: 16 rows of a member's squared window sum over the main
    // block's channels, 16 * tw * cn * 255^2, must stay below 2^32)
    int twMax = 0;
    for (const Bucket &b : f->buckets) twMax = std::max(twMax, b.tw);
    const size_t prefixRow = (size_t)(cnP == 4 ? 4 : stat_pitch(cnP)) * hpP;
    // CVM_STATS_EPILOGUE: fast-form buckets without regions of interest take
    // their window statistics from the frame's summed-area table inside the
    // inverse-rows epilogue (no statistics kernel, no den written and read
    // back) when every member's squared window sum can be restored from its
    // residue modulo 2^32: area * cn * 16256 < 2^32, cn up to the frame's
    // channels.
    std::vector<char> satUse(fg->bg.size(), 0);
    bool anySat = false, anyStatsKernel = false;
    for (size_t b = 0; b < fg->bg.size(); b++) {
        const FleetBucketGeom &bg = *fg->bg[b];
        bool ok = f->statsMode == CVM_STATS_EPILOGUE && bg.form == CVM_FORM_FAST && f->roi.empty() && (f->step == 4 || f->step == 1);
        for (int i : bg.members) {
            if (!ok) break;
            const cvm_matcher *m = f->ms[i];
            ok = (unsigned long long)m->w * m->h * (unsigned)cnP * 16256ull < (1ull << 32);
        }
        satUse[b] = ok;
        anySat |= ok;
        anyStatsKernel |= !ok;
    }
    const size_t alphaRow = cnP == 4 ? (size_t)2 * hpP : 0;
    const size_t satElems = anySat ? (size_t)(ph + 1) * (prefixRow + alphaRow) : 0;
    const size_t satBlkElems = anySat ? (size_t)((ph + 15) / 16 + 1) * prefixRow : 0;
    const bool blkOk = anyStatsKernel && 16ull * (unsigned)twMax * (cnP == 4 ? 3u : 1u) * 65025ull < (1ull << 32);
    const size_t blkElems = blkOk ? prefixRow * (size_t)(ph / 16) : 0;
    const size_t bytes = Arena::bytes(n, sizeof(DevParams)) + Arena::bytes(1, sizeof(DevFrame)) +
                         Arena::bytes(n, sizeof(int)) + Arena::bytes(prefixElems, sizeof(unsigned int)) +
                         (blkElems ? Arena::bytes(blkElems, sizeof(unsigned int)) : 0) +
                         (satElems ? Arena::bytes(satElems, sizeof(unsigned int)) +
                                         Arena::bytes(satBlkElems, sizeof(unsigned int))
                                   : 0) +
                         frameBytes + partBytes + waveBytes;
    // Overlapped waves (fast-form buckets, more than one wave in all): the
    // inverse rows of wave k run on the side stream beside the statistics
    // and columns of wave k + 1, so the waves alternate between two sets of
    // column output and den lanes.  (C4, 256 templates on 2560x1440: fast
    // 9.549 -> 9.429 ms; the mixed form's tensor-core rows and the exact
    // form measured slower overlapped, 10.83 -> 11.24 and 22.45 -> 22.70 ms,
    // so they keep their waves in sequence.)
    int nwaves = 0;
    bool allFast = true;
    for (size_t b = 0; b < fg->bg.size(); b++) {
        nwaves += ((int)fg->bg[b]->members.size() + wave[b] - 1) / wave[b];
        allFast = allFast && fg->bg[b]->form == CVM_FORM_FAST;
    }
    const bool overlap = f->overlapWaves && allFast && nwaves > 1;
    const size_t bytes2 = bytes + (overlap ? waveBytes : 0);
    PoolBuf buf;
    CVM_TRY(pool_alloc(buf, bytes2, st));
    Arena A;
    A.base = static_cast<char *>(buf.p);
    DevParams *P = A.take<DevParams>(n);
    DevFrame *F = A.take<DevFrame>(1);
    int *counters = A.take<int>(n);
    unsigned int *prefix = A.take<unsigned int>(prefixElems);
    unsigned int *prefixBlk = blkElems ? A.take<unsigned int>(blkElems) : nullptr;
    unsigned int *sat = satElems ? A.take<unsigned int>(satElems) : nullptr;
    unsigned int *satBlk = satElems ? A.take<unsigned int>(satBlkElems) : nullptr;
    char *frameBase = A.base + A.used;
    A.used += frameBytes;
    Partial *parts = reinterpret_cast<Partial *>(A.base + A.used);
    A.used += partBytes;
    char *waveBase[2] = {A.base + A.used, A.base + A.used + (overlap ? waveBytes : 0)};
    SideStream *ss = overlap ? &side_stream() : nullptr;
    int gw = 0;  // waves issued so far (all buckets): the set a wave uses is gw & 1
    // On every exit (an error return included) the caller's stream joins all
    // the side stream's queued rows before the workspace (declared above, so
    // released after this) returns to the pool in the caller's stream order.
    struct SideJoin {
        SideStream *ss;
        cudaStream_t st;
        ~SideJoin() {
            if (ss) {
                cudaEventRecord(ss->colsDone, ss->waveRows);
                cudaStreamWaitEvent(st, ss->colsDone, 0);
            }
        }
    } sideJoin{ss, st};
    CVM_CUDA(cudaMemcpyAsync(P, f->dP, n * sizeof(DevParams), cudaMemcpyDeviceToDevice, st));
    CVM_CUDA(cudaMemsetAsync(F, 0, sizeof(DevFrame), st));
    CVM_CUDA(cudaMemsetAsync(counters, 0, n * sizeof(int), st));
    CVM_CUDA(launch_prep(nullptr, 0, 0, 0, f->step, 0, f->step == 4 ? dParent : nullptr, pstride, pw, ph, P, n, 0, 0,
                         0, F, st));
    CVM_CUDA(launch_row_prefix(dParent, pstride, f->step, pw, ph, cnP, prefix, hpP, st));
    if (prefixBlk) CVM_CUDA(launch_vblock(prefix, prefixBlk, ph / 16, prefixRow, st));
    if (sat) {
        CVM_CUDA(launch_sat(prefix, ph, prefixRow, satBlk, sat, st));
        if (alphaRow)  // the (s3, alpha squares) block after the main one, in both
            CVM_CUDA(launch_sat(prefix + (size_t)ph * prefixRow, ph, alphaRow, satBlk, sat + (size_t)(ph + 1) * prefixRow,
                                st));
    }
    for (size_t b = 0; b < fg->bg.size(); b++) {
        const FleetBucketGeom &bg = *fg->bg[b];
        const Geom &G = bg.G;
        const bool fast = bg.form != CVM_FORM_EXACT;
        float2 *frame[2] = {nullptr, nullptr};
        float2 *scratch[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
        float2 *lanes[2] = {nullptr, nullptr};
        {
            Arena fa;
            fa.base = frameBase;
            for (int c = 0; c < G.nclass; c++) frame[c] = fa.take<float2>(spec_elems(G.fc[c], cnS));
            for (int set = 0; set < (overlap ? 2 : 1); set++) {
                Arena wa;
                wa.base = waveBase[set];
                for (int c = 0; c < G.nclass; c++)
                    scratch[set][c] = wa.take<float2>((size_t)wave[b] * bg.memberScratch[c]);
                lanes[set] = wa.take<float2>((size_t)wave[b] * bg.rwMax * bg.rhMax);
            }
        }
        // Phase 1: the frame's tile spectra, once per bucket (fleet.go:240-263).
        // the fast form transforms the frame offset by -128 (the zero-mean
        // templates make the correlation independent of the offset)
        const float off[4] = {128.f, 128.f, 128.f, 128.f};
        for (int c = 0; c < G.nclass; c++) {
            CVM_CUDA(launch_fwd_rows(dParent, pstride, f->step, cnS, &F->cnMax, G.g, G.fc[c], frame[c], cnS, st, 0,
                                     nullptr, 1.0f, fast ? off : nullptr));
            MemberSet none;
            memset(&none, 0, sizeof none);
            CVM_CUDA(launch_cols(0, frame[c], frame[c], cnS, G.g, G.fc[c], c, cnS, &F->cnMax, 1.0f, none, 1, st));
        }
        // Phase 2: member tails in waves (fleet.go:265-328).
        MemberSet ms;
        memset(&ms, 0, sizeof ms);
        ms.table = bg.table;
        ms.params = P;
        ms.lanes = lanes[0];
        ms.lanesStride = (size_t)bg.rwMax * bg.rhMax;
        ms.anyRoi = !f->roi.empty();
        ms.form = bg.form;
        if (satUse[b]) {
            ms.sat = sat;
            ms.satRow = prefixRow;
            ms.satAlpha = alphaRow ? (size_t)(ph + 1) * prefixRow : 0;
            ms.satNp = cnP == 4 ? 4 : 2;
        }
        for (int c = 0; c < G.nclass; c++) {
            ms.scratch[c] = scratch[0][c];
            ms.scratchStride[c] = bg.memberScratch[c];
        }
        const int nm = (int)bg.members.size();
        for (int w0 = 0; w0 < nm; w0 += wave[b], gw++) {
            const int nw = std::min(wave[b], nm - w0);
            const int set = overlap ? (gw & 1) : 0;
            // the set's previous wave (two waves back) has finished its rows
            if (overlap && gw >= 2) CVM_CUDA(cudaStreamWaitEvent(st, ss->rowsDone[set], 0));
            ms.lanes = lanes[set];
            for (int c = 0; c < G.nclass; c++) ms.scratch[c] = scratch[set][c];
            ms.first = w0;
            SepGrid sgP = bg.sg;
            sgP.hp = hpP;
            if (!satUse[b])
                CVM_CUDA(launch_sep_stats(dParent, pstride, f->step, pw, ph, ms, nw, 0, 0, sgP, f->step == 4 ? 3 : 1,
                                          cnP, prefix, 0, st, 1, nullptr, nullptr, prefixBlk));
            for (int c = 0; c < G.nclass; c++)
                CVM_CUDA(launch_cols(fast ? 3 : 2, frame[c], nullptr, cnS, G.g, G.fc[c], c, cnS, nullptr, 1.0f, ms, nw,
                                     st));
            cudaStream_t rst = st;
            if (overlap) {
                CVM_CUDA(cudaEventRecord(ss->colsDone, st));
                CVM_CUDA(cudaStreamWaitEvent(ss->waveRows, ss->colsDone, 0));
                rst = ss->waveRows;
            }
            for (int c = 0; c < G.nclass; c++)
                CVM_CUDA(launch_inv_rows(G.g, G.fc[c], c, fast ? 1 : cnS, ms, nw, G.fc[c].dftH, bg.partOff[c],
                                         bg.nparts, parts, counters, dOut, rst, fast));
            if (overlap) CVM_CUDA(cudaEventRecord(ss->rowsDone[set], rst));
        }
    }
    return CVM_OK;
}

}  // namespace

// ================================================================= C ABI

// ========================================================= frame streams

struct cvm_stream {
    cvm_fleet *color = nullptr, *gray = nullptr;
    int pw = 0, ph = 0;
    size_t pitch = 0, gpitch = 0;
    int nColor = 0, nGray = 0;
    cudaStream_t cs = nullptr;  // matching
    cudaStream_t gs = nullptr;  // the gray fleet, a branch forked from cs and joined back
    cudaStream_t xs = nullptr;  // frame uploads
    cudaEvent_t fork = nullptr, join = nullptr;
    struct Slot {
        uint8_t *hFrame = nullptr;   // page-locked staging
        uint8_t *dFrame = nullptr, *dGray = nullptr;
        cvm_result *dOut = nullptr;  // colour results then gray results
        cvm_result *hOut = nullptr;  // page-locked copy of dOut
        cudaGraphExec_t exec = nullptr;
        cudaEvent_t t0 = nullptr, copied = nullptr, done = nullptr;
        bool busy = false;
    } slot[2];
    int next = 0;          // slot of the next push
    int oldest = 0;        // slot of the next pull
    int inflight = 0;
    int graphed = 0;
    int launches = 0;
    ~cvm_stream() {
        for (Slot &sl : slot) {
            if (sl.busy && sl.done) cudaEventSynchronize(sl.done);
            if (sl.exec) cudaGraphExecDestroy(sl.exec);
            if (sl.hFrame) cudaFreeHost(sl.hFrame);
            if (sl.hOut) cudaFreeHost(sl.hOut);
            if (sl.dFrame) cudaFree(sl.dFrame);
            if (sl.dGray) cudaFree(sl.dGray);
            if (sl.dOut) cudaFree(sl.dOut);
            for (cudaEvent_t e : {sl.t0, sl.copied, sl.done})
                if (e) cudaEventDestroy(e);
        }
        if (cs) cudaStreamDestroy(cs);
        if (gs) cudaStreamDestroy(gs);
        if (xs) cudaStreamDestroy(xs);
        for (cudaEvent_t e : {fork, join})
            if (e) cudaEventDestroy(e);
    }
};

namespace {

// The per-frame pipeline of one slot on s->cs: the colour FindAll, and
// beside it on s->gs (forked from cs after the frame arrived, joined back
// before the results leave) the gray conversion and the gray FindAll --
// independent work (both read the frame, they write disjoint result
// ranges, each takes its workspace from the stream-ordered pool), so the
// gray fleet's short launches fill the colour fleet's launch tails; then
// the results back to page-locked memory.
int stream_pipeline(cvm_stream *s, cvm_stream::Slot &sl) {
    if (s->gray) {
        CVM_CUDA(cudaEventRecord(s->fork, s->cs));
        CVM_CUDA(cudaStreamWaitEvent(s->gs, s->fork, 0));
        CVM_CUDA(launch_gray(sl.dFrame, (long long)s->pitch, s->pw, s->ph, sl.dGray, (long long)s->gpitch, s->gs));
        CVM_TRY(fleet_find_dev(s->gray, sl.dGray, (long long)s->gpitch, s->pw, s->ph, sl.dOut + s->nColor, s->gs));
        CVM_CUDA(cudaEventRecord(s->join, s->gs));
    }
    CVM_TRY(fleet_find_dev(s->color, sl.dFrame, (long long)s->pitch, s->pw, s->ph, sl.dOut, s->cs));
    if (s->gray) CVM_CUDA(cudaStreamWaitEvent(s->cs, s->join, 0));
    CVM_CUDA(cudaMemcpyAsync(sl.hOut, sl.dOut, (size_t)(s->nColor + s->nGray) * sizeof(cvm_result),
                             cudaMemcpyDeviceToHost, s->cs));
    return CVM_OK;
}

// Capture the slot's pipeline as a graph.  The caches it reads (plans,
// member spectra) are built by an uncaptured run first.  On any capture
// failure the stream keeps issuing the pipeline launch by launch.
void stream_capture(cvm_stream *s, cvm_stream::Slot &sl) {
    if (cudaStreamBeginCapture(s->cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const uint64_t l0 = g_launches.load();
    const int rc = stream_pipeline(s, sl);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(s->cs, &g);
    if (rc != CVM_OK || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        return;
    }
    s->launches = (int)(g_launches.load() - l0);
    if (cudaGraphInstantiate(&sl.exec, g, 0) != cudaSuccess) {
        sl.exec = nullptr;
        cudaGetLastError();
    }
    cudaGraphDestroy(g);
}

}  // namespace

extern "C" {

size_t cvm_last_error(char *buf, size_t len) {
    const std::string &e = t_err;
    if (buf && len > 0) {
        const size_t c = e.size() < len - 1 ? e.size() : len - 1;
        memcpy(buf, e.data(), c);
        buf[c] = 0;
    }
    return e.size();
}

int cvm_match(const uint8_t *parent, int64_t pstride, int pw, int ph, const uint8_t *sub, int64_t sstride, int sw,
              int sh, cvm_result *out) {
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(check_image(sub, sw, sh));
    CVM_TRY(check_match_rgba(parent, pstride, pw, ph, sub, sstride, sw, sh));
    return host_solo(parent, pstride, pw, ph, sub, sstride, sw, sh, 1, 4, 4, 0, nullptr, out);
}

int cvm_match_map(const uint8_t *parent, int64_t pstride, int pw, int ph, const uint8_t *sub, int64_t sstride,
                  int sw, int sh, float *map) {
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(check_image(sub, sw, sh));
    CVM_TRY(check_match_rgba(parent, pstride, pw, ph, sub, sstride, sw, sh));
    if (!map) return fail(CVM_ERR_ARGS, "cvmatch_gpu: MatchMap needs a map buffer");
    cvm_result r;
    return host_solo(parent, pstride, pw, ph, sub, sstride, sw, sh, 1, 4, 4, 0, map, &r);
}

int cvm_match_map_peaks(const uint8_t *parent, int64_t pstride, int pw, int ph, const uint8_t *sub, int64_t sstride,
                        int sw, int sh, float thresh, int rx, int ry, int32_t *xy, int max_peaks, int32_t *count) {
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(check_image(sub, sw, sh));
    CVM_TRY(check_match_rgba(parent, pstride, pw, ph, sub, sstride, sw, sh));
    if (!count || max_peaks < 0 || (max_peaks > 0 && !xy) || rx < 0 || ry < 0 || ph - sh + 1 > 65535)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: bad occurrence request");
    cvm_result r;
    const PeakReq pk{thresh, rx, ry, xy, max_peaks, count};
    return host_solo(parent, pstride, pw, ph, sub, sstride, sw, sh, 1, 4, 4, 0, nullptr, &r, &pk);
}

int cvm_match_u8_peaks(const uint8_t *img, int64_t istride, int iw, int ih, const uint8_t *tpl, int64_t tstride,
                       int tw, int th, int cn, int step, float thresh, int rx, int ry, int32_t *xy, int max_peaks,
                       int32_t *count) {
    CVM_TRY(check_match_args(iw, ih, istride, tstride, tw, th, cn, step));
    if (!img || !tpl) return fail(CVM_ERR_NIL_IMAGE, "cvmatch: nil image");
    if (!count || max_peaks < 0 || (max_peaks > 0 && !xy) || rx < 0 || ry < 0 || ih - th + 1 > 65535)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: bad occurrence request");
    cvm_result r;
    const PeakReq pk{thresh, rx, ry, xy, max_peaks, count};
    return host_solo(img, istride, iw, ih, tpl, tstride, tw, th, 0, cn, step, 0, nullptr, &r, &pk);
}

int cvm_peaks_device(const float *d_map, int w, int h, float thresh, int rx, int ry, int32_t *d_xy, int max_peaks,
                     int32_t *d_count, void *stream) {
    if (!d_map || !d_count || w < 1 || h < 1 || h > 65535 || max_peaks < 0 || (max_peaks > 0 && !d_xy) || rx < 0 ||
        ry < 0)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: bad occurrence request");
    CVM_TRY(ensure_device());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    PoolBuf b;
    CVM_TRY(pool_alloc(b, peaks_scratch_ints(w, h) * sizeof(int), st));
    CVM_CUDA(launch_peaks(d_map, w, h, thresh, rx, ry, static_cast<int *>(b.p), d_xy, max_peaks, d_count, st));
    return CVM_OK;
}

int cvm_match_gray(const uint8_t *parent, int64_t pstride, int pw, int ph, const uint8_t *sub, int64_t sstride,
                   int sw, int sh, cvm_result *out) {
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(check_image(sub, sw, sh));
    CVM_TRY(check_match_args(pw, ph, pstride, sstride, sw, sh, 1, 1));
    return host_solo(parent, pstride, pw, ph, sub, sstride, sw, sh, 0, 1, 1, 0, nullptr, out);
}

int cvm_match_gray_rgba(const uint8_t *parent, int64_t pstride, int pw, int ph, const uint8_t *sub,
                        int64_t sstride, int sw, int sh, cvm_result *out) {
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(check_image(sub, sw, sh));
    if (pstride < (int64_t)pw * 4 || sstride < (int64_t)sw * 4)
        return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d, cn=1 step=1)", sw, sh, pw, ph);
    CVM_TRY(check_match_args(pw, ph, (int64_t)pw, (int64_t)sw, sw, sh, 1, 1));
    return host_solo(parent, pstride, pw, ph, sub, sstride, sw, sh, 0, 1, 1, 1, nullptr, out);
}

int cvm_match_u8(const uint8_t *img, int64_t istride, int iw, int ih, const uint8_t *tpl, int64_t tstride, int tw,
                 int th, int cn, int step, float *map, cvm_result *out) {
    CVM_TRY(check_match_args(iw, ih, istride, tstride, tw, th, cn, step));
    if (!img || !tpl) return fail(CVM_ERR_NIL_IMAGE, "cvmatch: nil image");
    return host_solo(img, istride, iw, ih, tpl, tstride, tw, th, 0, cn, step, 0, map, out);
}

int cvm_match_u8_device(const uint8_t *d_img, int64_t istride, int iw, int ih, const uint8_t *d_tpl,
                        int64_t tstride, int tw, int th, int cn, int step, float *d_map, cvm_result *d_out,
                        void *stream) {
    CVM_TRY(check_match_args(iw, ih, istride, tstride, tw, th, cn, step));
    CVM_TRY(ensure_device());
    SoloJob J;
    memset(&J, 0, sizeof J);
    J.form = solo_form();
    J.img = d_img;
    J.istride = istride;
    J.iw = iw;
    J.ih = ih;
    J.step = step;
    J.mode = 0;
    J.cnFixed = cn;
    J.tpl = d_tpl;
    J.tstride = tstride;
    J.tw = tw;
    J.th = th;
    J.map = d_map;
    J.out = d_out;
    return run_solo(J, static_cast<cudaStream_t>(stream));
}

int cvm_match_device(const uint8_t *d_parent, int64_t pstride, int pw, int ph, const uint8_t *d_sub,
                     int64_t sstride, int sw, int sh, float *d_map, cvm_result *d_out, void *stream) {
    CVM_TRY(check_image(d_parent, pw, ph));
    CVM_TRY(check_image(d_sub, sw, sh));
    CVM_TRY(check_match_args(pw, ph, pstride, sstride, sw, sh, 4, 4));
    CVM_TRY(ensure_device());
    SoloJob J;
    memset(&J, 0, sizeof J);
    J.form = solo_form();
    J.img = d_parent;
    J.istride = pstride;
    J.iw = pw;
    J.ih = ph;
    J.step = 4;
    J.mode = 1;
    J.cnFixed = 4;
    J.tpl = d_sub;
    J.tstride = sstride;
    J.tw = sw;
    J.th = sh;
    J.map = d_map;
    J.out = d_out;
    return run_solo(J, static_cast<cudaStream_t>(stream));
}

int cvm_rgba_to_gray(const uint8_t *pix, int64_t stride, int w, int h, uint8_t *out) {
    CVM_TRY(check_image(pix, w, h));
    if (stride < (int64_t)w * 4) return fail(CVM_ERR_ARGS, "cvmatch_gpu: stride below width*4");
    CVM_TRY(ensure_device());
    cudaStream_t st = thread_stream();
    PoolBuf bi, bo;
    long long ip;
    CVM_TRY(upload_image(bi, pix, stride, w, h, 4, &ip, st));
    CVM_TRY(pool_alloc(bo, (size_t)w * h, st));
    CVM_CUDA(launch_gray(static_cast<const uint8_t *>(bi.p), ip, w, h, static_cast<uint8_t *>(bo.p), w, st));
    CVM_CUDA(cudaMemcpyAsync(out, bo.p, (size_t)w * h, cudaMemcpyDeviceToHost, st));
    CVM_CUDA(cudaStreamSynchronize(st));
    return CVM_OK;
}

int cvm_rgba_to_gray_device(const uint8_t *d_pix, int64_t stride, int w, int h, uint8_t *d_out, int64_t ostride,
                            void *stream) {
    CVM_TRY(check_image(d_pix, w, h));
    if (!d_out) return fail(CVM_ERR_NIL_IMAGE, "cvmatch: nil image");
    if (stride < (int64_t)w * 4 || ostride < (int64_t)w)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: stride below width*4, or output stride below width");
    CVM_TRY(ensure_device());
    CVM_CUDA(launch_gray(d_pix, stride, w, h, d_out, ostride, static_cast<cudaStream_t>(stream)));
    return CVM_OK;
}

int cvm_alpha_const(const uint8_t *pix, int64_t stride, int w, int h, int *out) {
    CVM_TRY(check_image(pix, w, h));
    if (stride < (int64_t)w * 4) return fail(CVM_ERR_ARGS, "cvmatch_gpu: stride below width*4");
    CVM_TRY(ensure_device());
    cudaStream_t st = thread_stream();
    PoolBuf bi, bf;
    long long ip;
    CVM_TRY(upload_image(bi, pix, stride, w, h, 4, &ip, st));
    CVM_TRY(pool_alloc(bf, sizeof(unsigned int), st));
    CVM_CUDA(cudaMemsetAsync(bf.p, 0, sizeof(unsigned int), st));
    CVM_CUDA(launch_alpha_scan(static_cast<const uint8_t *>(bi.p), ip, w, h, static_cast<unsigned int *>(bf.p), st));
    unsigned int mism = 0;
    CVM_CUDA(cudaMemcpyAsync(&mism, bf.p, sizeof mism, cudaMemcpyDeviceToHost, st));
    CVM_CUDA(cudaStreamSynchronize(st));
    *out = mism == 0;
    return CVM_OK;
}

int cvm_matcher_new(const uint8_t *pix, int64_t stride, int w, int h, int step, cvm_matcher **out) {
    CVM_TRY(check_image(pix, w, h));
    if (step != 1 && step != 4) return fail(CVM_ERR_ARGS, "cvmatch_gpu: matcher step must be 1 or 4");
    if (stride < (int64_t)w * step) return fail(CVM_ERR_ARGS, "cvmatch_gpu: stride below width*step");
    if ((int64_t)w * h > stats_cap(step))
        return fail(CVM_ERR_STATS_CAP, "cvmatch: template area %dx%d exceeds the exact-statistics bound", w, h);
    CVM_TRY(ensure_device());
    std::unique_ptr<cvm_matcher> m(new cvm_matcher());
    m->w = w;
    m->h = h;
    m->step = step;
    // Exact statistics over step channels (matcher.go:75) and the template
    // alpha scan (matcher.go:49).
    const int64_t area = (int64_t)w * h;
    bool aconst = true;
    for (int k = 0; k < step; k++) {
        int64_t s = 0, s2 = 0;
        for (int y = 0; y < h; y++) {
            const uint8_t *row = pix + (int64_t)y * stride + k;
            for (int x = 0; x < w; x++) {
                const int64_t v = row[(int64_t)x * step];
                s += v;
                s2 += v * v;
            }
        }
        m->tsum[k] = s;
        m->varSum += area * s2 - s * s;
    }
    if (step == 4)
        for (int y = 0; y < h && aconst; y++)
            for (int x = 0; x < w; x++)
                if (pix[(int64_t)y * stride + 4 * x + 3] != pix[3]) {
                    aconst = false;
                    break;
                }
    m->aConst = aconst;
    cudaStream_t st = thread_stream();
    CVM_CUDA(cudaMalloc(&m->dPix, (size_t)w * h * step));
    CVM_CUDA(cudaMemcpy2DAsync(m->dPix, (size_t)w * step, pix, (size_t)stride, (size_t)w * step, h,
                               cudaMemcpyHostToDevice, st));
    // Raw template sums (and the template's alpha flag) through the same
    // statistics kernel one-shot calls use; a scratch frame record serves
    // the kernel's finalisation, which Find repeats per frame.
    CVM_CUDA(cudaMalloc(&m->dP, sizeof(DevParams)));
    PoolBuf fb;
    CVM_TRY(pool_alloc(fb, sizeof(DevFrame), st));
    CVM_CUDA(cudaMemsetAsync(m->dP, 0, sizeof(DevParams), st));
    CVM_CUDA(cudaMemsetAsync(fb.p, 0, sizeof(DevFrame), st));
    CVM_CUDA(launch_prep(m->dPix, (long long)w * step, w, h, step, step, nullptr, 0, 0, 0, m->dP, 1, 1,
                         step == 4 ? 1 : 0, step == 4 ? 4 : 1, static_cast<DevFrame *>(fb.p), st));
    CVM_CUDA(cudaStreamSynchronize(st));
    *out = m.release();
    return CVM_OK;
}

int cvm_matcher_find(cvm_matcher *m, const uint8_t *parent, int64_t pstride, int pw, int ph, cvm_result *out) {
    if (!m) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil matcher");
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(ensure_device());
    if (m->w > pw || m->h > ph)
        return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d)", m->w, m->h, pw, ph);
    if (m->varSum == 0) {
        *out = kFlatResult;
        return CVM_OK;
    }
    cudaStream_t st = thread_stream();
    PoolBuf bi, bo;
    long long ip;
    CVM_TRY(upload_image(bi, parent, pstride, pw, ph, m->step, &ip, st));
    CVM_TRY(pool_alloc(bo, sizeof(cvm_result), st));
    CVM_TRY(matcher_find_dev(m, static_cast<const uint8_t *>(bi.p), ip, pw, ph, static_cast<cvm_result *>(bo.p), st));
    CVM_CUDA(cudaMemcpyAsync(out, bo.p, sizeof(cvm_result), cudaMemcpyDeviceToHost, st));
    CVM_CUDA(cudaStreamSynchronize(st));
    return CVM_OK;
}

int cvm_matcher_find_device(cvm_matcher *m, const uint8_t *d_parent, int64_t pstride, int pw, int ph,
                            cvm_result *d_out, void *stream) {
    if (!m) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil matcher");
    CVM_TRY(check_image(d_parent, pw, ph));
    CVM_TRY(ensure_device());
    return matcher_find_dev(m, d_parent, pstride, pw, ph, d_out, static_cast<cudaStream_t>(stream));
}

void cvm_matcher_free(cvm_matcher *m) { delete m; }

int cvm_fleet_new(cvm_matcher *const *ms, int n, cvm_fleet **out) {
    if (n <= 0 || !ms) return fail(CVM_ERR_EMPTY_FLEET, "cvmatch: empty fleet");
    CVM_TRY(ensure_device());
    std::unique_ptr<cvm_fleet> f(new cvm_fleet());
    f->ms.assign(ms, ms + n);
    f->step = ms[0]->step;
    for (cvm_matcher *m : f->ms)
        if (m->step != f->step) return fail(CVM_ERR_MIXED_FLEET, "cvmatch: fleet mixes color and gray matchers");
    std::vector<MemberShape> shapes;
    for (cvm_matcher *m : f->ms) shapes.push_back(MemberShape{m->w, m->h, m->varSum == 0});
    f->buckets = bucketize(shapes);
    CVM_CUDA(cudaMalloc(&f->dP, n * sizeof(DevParams)));
    for (int i = 0; i < n; i++)
        CVM_CUDA(cudaMemcpy(f->dP + i, f->ms[i]->dP, sizeof(DevParams), cudaMemcpyDeviceToDevice));
    *out = f.release();
    return CVM_OK;
}

int cvm_fleet_find_all(cvm_fleet *f, const uint8_t *parent, int64_t pstride, int pw, int ph, cvm_result *out) {
    if (!f) return fail(CVM_ERR_EMPTY_FLEET, "cvmatch: empty fleet");
    CVM_TRY(check_image(parent, pw, ph));
    CVM_TRY(ensure_device());
    const int n = (int)f->ms.size();
    for (int i = 0; i < n; i++)
        if (f->ms[i]->w > pw || f->ms[i]->h > ph)
            return fail(CVM_ERR_ARGS, "cvmatch: bad match arguments (%dx%d in %dx%d)", f->ms[i]->w, f->ms[i]->h, pw,
                        ph);
    cudaStream_t st = thread_stream();
    PoolBuf bi, bo;
    long long ip;
    CVM_TRY(upload_image(bi, parent, pstride, pw, ph, f->step, &ip, st));
    CVM_TRY(pool_alloc(bo, n * sizeof(cvm_result), st));
    CVM_TRY(fleet_find_dev(f, static_cast<const uint8_t *>(bi.p), ip, pw, ph, static_cast<cvm_result *>(bo.p), st));
    CVM_CUDA(cudaMemcpyAsync(out, bo.p, n * sizeof(cvm_result), cudaMemcpyDeviceToHost, st));
    CVM_CUDA(cudaStreamSynchronize(st));
    return CVM_OK;
}

int cvm_fleet_find_all_device(cvm_fleet *f, const uint8_t *d_parent, int64_t pstride, int pw, int ph,
                              cvm_result *d_out, void *stream) {
    if (!f) return fail(CVM_ERR_EMPTY_FLEET, "cvmatch: empty fleet");
    CVM_TRY(check_image(d_parent, pw, ph));
    CVM_TRY(ensure_device());
    return fleet_find_dev(f, d_parent, pstride, pw, ph, d_out, static_cast<cudaStream_t>(stream));
}

void cvm_fleet_free(cvm_fleet *f) { delete f; }

int cvm_set_autotune(int on) { return g_autotune.exchange(on ? 1 : 0); }

size_t cvm_autotune_report(char *buf, size_t len) {
    std::string j = "[";
    {
        std::lock_guard<std::mutex> lk(g_tuneMu);
        bool first = true;
        for (const auto &kv : g_tune) {
            const TuneKey &k = kv.first;
            const TuneEntry &e = kv.second;
            char b[256];
            snprintf(b, sizeof b,
                     "%s{\"frame\":[%d,%d],\"template\":[%d,%d],\"mode\":%d,\"cn\":%d,\"step\":%d,\"form\":%d,"
                     "\"plan\":[%d,%d],\"candidates\":[",
                     first ? "" : ",", k.iw, k.ih, k.tw, k.th, k.mode, k.cn, k.step, k.form, e.plan.dftW, e.plan.dftH);
            j += b;
            for (int i = 0; i < e.n; i++) {
                snprintf(b, sizeof b, "%s{\"plan\":[%d,%d],\"ms\":%.5f}", i ? "," : "", e.cand[i].dftW, e.cand[i].dftH,
                         (double)e.ms[i]);
                j += b;
            }
            j += "]}";
            first = false;
        }
        for (const auto &kv : g_fleetTune) {
            const FleetTuneKey &k = kv.first;
            const FleetTuneEntry &e = kv.second;
            char b[256];
            snprintf(b, sizeof b,
                     "%s{\"fleet\":true,\"frame\":[%d,%d],\"bucket\":[%d,%d],\"members\":%d,\"step\":%d,"
                     "\"form\":%d,\"plan\":[%d,%d],\"candidates\":[",
                     first ? "" : ",", k.pw, k.ph, k.tw, k.th, k.n, k.step, k.form, e.plan.dftW, e.plan.dftH);
            j += b;
            for (int i = 0; i < e.n; i++) {
                snprintf(b, sizeof b, "%s{\"plan\":[%d,%d],\"ms_per_member\":%.5f,\"ms_shared\":%.5f,\"ms\":%.5f}",
                         i ? "," : "", e.cand[i].dftW, e.cand[i].dftH, (double)e.perMember[i], (double)e.shared[i],
                         (double)e.total[i]);
                j += b;
            }
            j += "]}";
            first = false;
        }
    }
    j += "]";
    if (buf && len) {
        const size_t n = j.size() < len - 1 ? j.size() : len - 1;
        memcpy(buf, j.data(), n);
        buf[n] = 0;
    }
    return j.size();
}

int cvm_set_form(int form) {
    if (form != CVM_FORM_EXACT && form != CVM_FORM_FAST && form != CVM_FORM_MIXED)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: unknown form %d", form);
    g_soloForm.store(form, std::memory_order_relaxed);
    return CVM_OK;
}

int cvm_get_form(void) { return solo_form(); }

int cvm_tc_selftest(double *dft_err, double *gemm_err) {
    CVM_TRY(ensure_device());
    double a = 0, b = 0;
    CVM_CUDA(tc_selftest(&a, &b));
    if (dft_err) *dft_err = a;
    if (gemm_err) *gemm_err = b;
    return CVM_OK;
}

int cvm_device_status(int *tc_timeouts) {
    CVM_TRY(ensure_device());
    const int v = tc_error_read_clear(), w = rows_error_read_clear();
    if (v < 0 || w < 0) return fail(CVM_ERR_CUDA, "cvmatch_gpu: reading the device status failed");
    if (tc_timeouts) *tc_timeouts = v | w;
    return CVM_OK;
}

int cvm_fleet_set_form(cvm_fleet *f, int form) {
    if (!f) return fail(CVM_ERR_EMPTY_FLEET, "cvmatch: empty fleet");
    if (form != CVM_FORM_EXACT && form != CVM_FORM_FAST && form != CVM_FORM_MIXED)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: unknown fleet form %d", form);
    std::lock_guard<std::mutex> lk(f->mu);
    if (f->form != form) {
        f->form = form;
        f->geom.reset();  // spectra of the other form
    }
    return CVM_OK;
}

int cvm_fleet_set_roi(cvm_fleet *f, int member, int x, int y, int w, int h) {
    if (!f) return fail(CVM_ERR_EMPTY_FLEET, "cvmatch: empty fleet");
    const int n = (int)f->ms.size();
    if (member < 0 || member >= n) return fail(CVM_ERR_ARGS, "cvmatch_gpu: fleet member %d of %d", member, n);
    std::lock_guard<std::mutex> lk(f->mu);
    if (f->roi.empty()) f->roi.assign(4 * (size_t)n, 0);
    f->roi[4 * member] = x;
    f->roi[4 * member + 1] = y;
    f->roi[4 * member + 2] = w;
    f->roi[4 * member + 3] = h;
    f->roiGen++;
    return CVM_OK;
}

int cvm_stream_new(cvm_fleet *color, cvm_fleet *gray, int pw, int ph, cvm_stream **out) {
    if (!out) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil output handle");
    *out = nullptr;
    if (!color || color->ms.empty()) return fail(CVM_ERR_EMPTY_FLEET, "cvmatch: empty fleet");
    if (color->step != 4) return fail(CVM_ERR_MIXED_FLEET, "cvmatch_gpu: the colour fleet of a stream must be RGBA");
    if (gray && (gray->ms.empty() || gray->step != 1))
        return fail(CVM_ERR_MIXED_FLEET, "cvmatch_gpu: the gray fleet of a stream must hold gray matchers");
    if (pw < 1 || ph < 1) return fail(CVM_ERR_EMPTY_IMAGE, "cvmatch: empty image");
    CVM_TRY(ensure_device());
    auto s = std::make_unique<cvm_stream>();
    s->color = color;
    s->gray = gray;
    s->pw = pw;
    s->ph = ph;
    s->pitch = align_up((size_t)pw * 4, 128);
    s->gpitch = align_up((size_t)pw, 128);
    s->nColor = (int)color->ms.size();
    s->nGray = gray ? (int)gray->ms.size() : 0;
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    CVM_CUDA(cudaStreamCreateWithFlags(&s->cs, cudaStreamNonBlocking));
    CVM_CUDA(cudaStreamCreateWithFlags(&s->gs, cudaStreamNonBlocking));
    CVM_CUDA(cudaStreamCreateWithPriority(&s->xs, cudaStreamNonBlocking, greatest));
    CVM_CUDA(cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming));
    CVM_CUDA(cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming));
    const size_t nres = (size_t)(s->nColor + s->nGray);
    for (cvm_stream::Slot &sl : s->slot) {
        CVM_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&sl.hFrame), s->pitch * ph, cudaHostAllocDefault));
        CVM_CUDA(cudaHostAlloc(reinterpret_cast<void **>(&sl.hOut), nres * sizeof(cvm_result), cudaHostAllocDefault));
        CVM_CUDA(cudaMalloc(&sl.dFrame, s->pitch * ph));
        if (gray) CVM_CUDA(cudaMalloc(&sl.dGray, s->gpitch * ph));
        CVM_CUDA(cudaMalloc(&sl.dOut, nres * sizeof(cvm_result)));
        CVM_CUDA(cudaEventCreate(&sl.t0));
        CVM_CUDA(cudaEventCreate(&sl.copied));
        CVM_CUDA(cudaEventCreate(&sl.done));
        CVM_CUDA(cudaMemsetAsync(sl.dFrame, 0, s->pitch * ph, s->cs));
    }
    // build the fleets' caches for this frame size, then capture each slot
    CVM_TRY(stream_pipeline(s.get(), s->slot[0]));
    CVM_CUDA(cudaStreamSynchronize(s->cs));
    for (cvm_stream::Slot &sl : s->slot) stream_capture(s.get(), sl);
    s->graphed = s->slot[0].exec && s->slot[1].exec;
    if (!s->graphed) {
        for (cvm_stream::Slot &sl : s->slot)
            if (sl.exec) {
                cudaGraphExecDestroy(sl.exec);
                sl.exec = nullptr;
            }
    }
    *out = s.release();
    return CVM_OK;
}

int cvm_stream_push(cvm_stream *s, const uint8_t *rgba, int64_t stride) {
    if (!s) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil stream");
    if (!rgba) return fail(CVM_ERR_NIL_IMAGE, "cvmatch: nil image");
    if (stride < (int64_t)s->pw * 4) return fail(CVM_ERR_ARGS, "cvmatch_gpu: stride below width*4");
    if (s->inflight == 2) return fail(CVM_ERR_ARGS, "cvmatch_gpu: two frames in flight; pull one first");
    cvm_stream::Slot &sl = s->slot[s->next];
    // the slot's previous upload has left the staging buffer (its frame was pulled)
    CVM_CUDA(cudaEventSynchronize(sl.copied));
    const size_t row = (size_t)s->pw * 4;
    for (int y = 0; y < s->ph; y++) memcpy(sl.hFrame + (size_t)y * s->pitch, rgba + (size_t)y * stride, row);
    CVM_CUDA(cudaEventRecord(sl.t0, s->xs));
    CVM_CUDA(cudaMemcpyAsync(sl.dFrame, sl.hFrame, s->pitch * s->ph, cudaMemcpyHostToDevice, s->xs));
    CVM_CUDA(cudaEventRecord(sl.copied, s->xs));
    CVM_CUDA(cudaStreamWaitEvent(s->cs, sl.copied, 0));
    if (s->graphed)
        CVM_CUDA(cudaGraphLaunch(sl.exec, s->cs));
    else
        CVM_TRY(stream_pipeline(s, sl));
    CVM_CUDA(cudaEventRecord(sl.done, s->cs));
    sl.busy = true;
    s->next ^= 1;
    s->inflight++;
    return CVM_OK;
}

int cvm_stream_pull(cvm_stream *s, cvm_result *color_out, cvm_result *gray_out, double *device_ms) {
    if (!s) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil stream");
    if (s->inflight == 0) return fail(CVM_ERR_ARGS, "cvmatch_gpu: no frame in flight");
    cvm_stream::Slot &sl = s->slot[s->oldest];
    CVM_CUDA(cudaEventSynchronize(sl.done));
    if (color_out) memcpy(color_out, sl.hOut, (size_t)s->nColor * sizeof(cvm_result));
    if (gray_out && s->nGray) memcpy(gray_out, sl.hOut + s->nColor, (size_t)s->nGray * sizeof(cvm_result));
    if (device_ms) {
        float ms = 0;
        CVM_CUDA(cudaEventElapsedTime(&ms, sl.t0, sl.done));
        *device_ms = ms;
    }
    sl.busy = false;
    s->oldest ^= 1;
    s->inflight--;
    return CVM_OK;
}

int cvm_stream_info(cvm_stream *s, int *graphed, int *launches) {
    if (!s) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil stream");
    if (graphed) *graphed = s->graphed;
    if (launches) *launches = s->launches;
    return CVM_OK;
}

void cvm_stream_free(cvm_stream *s) { delete s; }

int cvm_plan(int tw, int th, int rw, int rh, int32_t out[6]) {
    if (tw < 1 || th < 1 || rw < 1 || rh < 1 || !out)
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: plan needs positive template and result sizes");
    const Plan p = make_plan(tw, th, rw, rh);
    out[0] = p.dftW;
    out[1] = p.dftH;
    out[2] = p.blockW;
    out[3] = p.blockH;
    out[4] = shrink_dh(p, rh, th);
    out[5] = ((rw + p.blockW - 1) / p.blockW) * ((rh + p.blockH - 1) / p.blockH);
    return CVM_OK;
}

int cvm_fleet_buckets(const cvm_fleet *f, int pw, int ph, int32_t *out, int cap) {
    if (!f) return -fail(CVM_ERR_ARGS, "cvmatch_gpu: nil fleet");
    const int nb = (int)f->buckets.size();
    for (int b = 0; b < nb && b < cap && out; b++) {
        const Bucket &bk = f->buckets[b];
        const int rw = pw - bk.tw + 1, rh = ph - bk.th + 1;
        int32_t *o = out + 9 * b;
        if (rw < 1 || rh < 1) {
            for (int k = 0; k < 9; k++) o[k] = 0;
            continue;
        }
        const Plan p = make_plan(bk.tw, bk.th, rw, rh);
        o[0] = bk.tw;
        o[1] = bk.th;
        o[2] = p.dftW;
        o[3] = p.dftH;
        o[4] = p.blockW;
        o[5] = p.blockH;
        o[6] = shrink_dh(p, rh, bk.th);
        o[7] = ((rw + p.blockW - 1) / p.blockW) * ((rh + p.blockH - 1) / p.blockH);
        o[8] = (int32_t)bk.members.size();
    }
    return nb;
}

int cvm_fleet_set_wave(cvm_fleet *f, int members) {
    if (!f || members < 0) return fail(CVM_ERR_ARGS, "cvmatch_gpu: bad wave size");
    f->waveMembers = members;
    return CVM_OK;
}

int cvm_fleet_set_overlap(cvm_fleet *f, int on) {
    if (!f) return fail(CVM_ERR_ARGS, "cvmatch_gpu: nil fleet");
    f->overlapWaves = on ? 1 : 0;
    return CVM_OK;
}

int cvm_fleet_set_stats(cvm_fleet *f, int mode) {
    if (!f || (mode != CVM_STATS_KERNEL && mode != CVM_STATS_EPILOGUE))
        return fail(CVM_ERR_ARGS, "cvmatch_gpu: bad statistics mode");
    f->statsMode = mode;
    return CVM_OK;
}

int cvm_fleet_bucket_members(const cvm_fleet *f, int b, int32_t *out, int cap) {
    if (!f || b < 0 || b >= (int)f->buckets.size()) return -fail(CVM_ERR_ARGS, "cvmatch_gpu: no such bucket");
    const std::vector<int> &m = f->buckets[b].members;
    for (int i = 0; i < (int)m.size() && i < cap && out; i++) out[i] = m[i];
    return (int)m.size();
}

void *cvm_host_alloc(size_t bytes) {
    void *p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
    return p;
}

void cvm_host_free(void *p) {
    if (p) cudaFreeHost(p);
}

uint64_t cvm_launch_count(void) { return g_launches.load(); }

void cvm_profile_enable(int on) { profile_enable(on); }

int cvm_profile_read(int i, char *name, size_t len, double *ms_total, uint64_t *launches) {
    unsigned long long n = 0;
    const int rc = profile_read(i, name, len, ms_total, &n);
    if (rc == 0 && launches) *launches = n;
    return rc;
}

int cvm_profile_span(int i, char *name, size_t len, double *t0_ms, double *t1_ms) {
    double a = 0, b = 0;
    const int rc = profile_span(i, name, len, &a, &b);
    if (rc == 0) {
        if (t0_ms) *t0_ms = a;
        if (t1_ms) *t1_ms = b;
    }
    return rc;
}

const char *cvm_version(void) { return "cvmatch_gpu 0.1 (sm_103a, reference-exact FP32 radix-4)"; }

}  // extern "C"
