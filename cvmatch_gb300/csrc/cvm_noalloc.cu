// cvm_noalloc.cu -- matchU8 on device buffers with no device allocation.
//
// Some callers cannot call cudaMalloc: code running inside a memory
// budget that another allocator owns (a framework's caching pool, a
// graphics or inference runtime that reserves the device at start-up), or
// real-time loops where a driver allocation's latency is not acceptable.
// This entry point serves them: its whole workspace -- spectra, the raw
// correlation, statistics, partial extrema and the twiddle tables -- lives
// in one file-scope device array of fixed size that every GPU loading the
// library holds until the process exits.  The caller still passes the
// image, the template and the outputs.
//
// It computes the exact form (the reference's float32 op sequence, bit
// for bit) whatever cvm_set_form selects: the fast form's statistics
// kernels need per-row window sums sized by the frame, which this fixed
// budget does not hold for the frames it accepts.
//
// Every call shares that array and it keeps the last call's contents;
// everything that must start at zero is cleared by each call.  Calls whose
// work overlaps on the GPU (several host threads, or several streams)
// race on the shared array: serialise them.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "cvm_internal.h"
#include "cvm_plan.h"

namespace cvm {
namespace {

// Fixed device scratch: twiddle tables for every transform size up to
// 2^14 (about 256 KB) followed by the per-call workspace.
constexpr size_t kNoAllocBytes = size_t(64) << 20;
constexpr int kMaxLog2 = 14;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

struct NoAllocDevice {
    bool ready = false;
    int status = CVM_OK;
    unsigned char *base = nullptr;  // device address of g_noalloc_scratch on this device
    size_t triOff[kMaxLog2 + 1] = {};
    size_t workOff = 0;
    int smemOptin = 0;              // largest opt-in dynamic shared memory per block
};

std::mutex g_noalloc_mu;
NoAllocDevice g_noalloc_dev[64];

int na_fail(int code, const char *msg) {
    set_error_message(msg);
    return code;
}

size_t up256(size_t v) { return (v + 255) / 256 * 256; }

// Set-up, once per device with that device current: resolve the array's
// device address and upload the twiddle tables (synchronous copies).
int noalloc_setup(NoAllocDevice **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return na_fail(CVM_ERR_NO_DEVICE, "cvmatch_gpu: no current CUDA device");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (d.ready) {
        *out = &d;
        return CVM_OK;
    }
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (major != 10 || minor != 3) return na_fail(CVM_ERR_NO_DEVICE, "cvmatch_gpu: built for sm_103a");
    cudaDeviceGetAttribute(&d.smemOptin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
        char b[200];
        snprintf(b, sizeof b, "cvmatch_gpu: cudaGetSymbolAddress(device scratch) failed: %s", cudaGetErrorString(e));
        return na_fail(CVM_ERR_CUDA, b);
    }
    d.base = static_cast<unsigned char *>(p);
    size_t off = 0;
    for (int l = 1; l <= kMaxLog2; l++) {
        std::vector<float> t = tri_twiddles(1 << l);
        if (t.empty()) t.assign(2, 0.f);
        d.triOff[l] = off;
        if (cudaMemcpy(d.base + off, t.data(), t.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
            return na_fail(CVM_ERR_CUDA, "cvmatch_gpu: uploading the twiddle tables to the device scratch failed");
        off = up256(off + t.size() * sizeof(float));
    }
    d.workOff = off;
    d.ready = true;
    *out = &d;
    return CVM_OK;
}

}  // namespace
}  // namespace cvm

using namespace cvm;

extern "C" int cvm_match_u8_device_noalloc(const uint8_t *d_img, int64_t istride, int iw, int ih,
                                           const uint8_t *d_tpl, int64_t tstride, int tw, int th, int cn,
                                           int step, float *d_map, cvm_result *d_out, void *stream) {
    if (cn < 1 || cn > 4 || step < cn || tw < 1 || th < 1 || tw > iw || th > ih || istride < (int64_t)iw * step ||
        tstride < (int64_t)tw * step) {
        char b[160];
        snprintf(b, sizeof b, "cvmatch: bad match arguments (%dx%d in %dx%d, cn=%d step=%d)", tw, th, iw, ih, cn, step);
        return na_fail(CVM_ERR_ARGS, b);
    }
    if ((int64_t)tw * th > stats_cap(cn)) {
        char b[160];
        snprintf(b, sizeof b, "cvmatch: template area %dx%d exceeds the exact-statistics bound for cn=%d", tw, th, cn);
        return na_fail(CVM_ERR_STATS_CAP, b);
    }
    if (!d_img || !d_tpl || !d_out) return na_fail(CVM_ERR_NIL_IMAGE, "cvmatch: nil image");
    NoAllocDevice *D = nullptr;
    int rc = noalloc_setup(&D);
    if (rc != CVM_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rw = iw - tw + 1, rh = ih - th + 1;

    // Geometry (newGoPlan + shrinkDH) with twiddles from the fixed tables.
    const Plan p = make_plan(tw, th, rw, rh);
    if (p.dftW > 8192 || p.dftH > 16384) return na_fail(CVM_ERR_UNSUPPORTED, "cvmatch_gpu: tile transform too large");
    const int dh2 = shrink_dh(p, rh, th);
    TileGeom g;
    g.ntx = (rw + p.blockW - 1) / p.blockW;
    g.nty = (rh + p.blockH - 1) / p.blockH;
    g.blockW = p.blockW;
    g.blockH = p.blockH;
    g.rwT = rw;
    g.rhT = rh;
    g.twL = tw;
    g.thL = th;
    g.tileFirst = 0;
    const int ntiles = g.ntx * g.nty;
    const int nclass = dh2 > 0 ? 2 : 1;
    FftClass fc[2];
    for (int c = 0; c < nclass; c++) {
        FftClass &f = fc[c];
        f.n = p.dftW;
        f.log2n = ilog2(p.dftW);
        f.hw = p.hw;
        f.hwp = (int)((p.hw + 15) / 16 * 16);
        f.dftH = c == 0 ? p.dftH : dh2;
        f.log2H = ilog2(f.dftH);
        f.triW = reinterpret_cast<const float2 *>(D->base + D->triOff[f.log2n]);
        f.triH = reinterpret_cast<const float2 *>(D->base + D->triOff[f.log2H]);
        f.tileFirst = nclass == 1 ? 0 : (c == 0 ? 0 : ntiles - g.ntx);
        f.ntiles = nclass == 1 ? ntiles : (c == 0 ? ntiles - g.ntx : g.ntx);
    }
    const NormGrid ng = norm_grid(rw, rh, tw, cn);
    const int nparts = ng.ncx * ng.nby;
    // The normalisation stages a window row of (128 + tw - 1) pixels per
    // result row group in shared memory; a very wide template needs more
    // than one block can have.  Refuse before anything is queued.
    if (ng.smemBytes > (size_t)D->smemOptin) {
        char b[220];
        snprintf(b, sizeof b,
                 "cvmatch_gpu: a %d-pixel-wide template needs %zu bytes of shared memory per block in the "
                 "fixed-scratch normalisation; the device allows %d (use cvm_match_u8_device)",
                 tw, ng.smemBytes, D->smemOptin);
        return na_fail(CVM_ERR_UNSUPPORTED, b);
    }

    // Workspace carved from the fixed array.
    size_t off = D->workOff;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = up256(off + bytes);
        return D->base + o;
    };
    DevParams *P = reinterpret_cast<DevParams *>(take(sizeof(DevParams)));
    DevFrame *F = reinterpret_cast<DevFrame *>(take(sizeof(DevFrame)));
    Partial *parts = reinterpret_cast<Partial *>(take((size_t)nparts * sizeof(Partial)));
    float *corr = d_map ? d_map : reinterpret_cast<float *>(take((size_t)rw * rh * sizeof(float)));
    float2 *spec[2] = {nullptr, nullptr}, *ts[2] = {nullptr, nullptr};
    for (int c = 0; c < nclass; c++) {
        spec[c] = reinterpret_cast<float2 *>(take((size_t)fc[c].ntiles * cn * fc[c].dftH * fc[c].hwp * sizeof(float2)));
        ts[c] = reinterpret_cast<float2 *>(take((size_t)cn * fc[c].dftH * fc[c].hwp * sizeof(float2)));
    }
    if (off > kNoAllocBytes) {
        char b[200];
        snprintf(b, sizeof b,
                 "cvmatch_gpu: this match needs %zu bytes of workspace; the fixed device scratch holds %zu "
                 "(use cvm_match_u8_device)",
                 off, kNoAllocBytes);
        return na_fail(CVM_ERR_UNSUPPORTED, b);
    }

#define NA_CUDA(call)                                                                          \
    do {                                                                                       \
        const cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                               \
            char b_[200];                                                                      \
            snprintf(b_, sizeof b_, "cvmatch_gpu: %s failed: %s", #call, cudaGetErrorString(e_)); \
            return na_fail(CVM_ERR_CUDA, b_);                                                  \
        }                                                                                      \
    } while (0)

    // The statistics and counters must start at zero on every call.
    NA_CUDA(cudaMemsetAsync(P, 0, sizeof(DevParams), st));
    NA_CUDA(cudaMemsetAsync(F, 0, sizeof(DevFrame), st));
    NA_CUDA(launch_prep(d_tpl, tstride, tw, th, step, cn, nullptr, 0, 0, 0, P, 1, 1, 0, cn, F, st));
    // Template spectrum on the main plan, scaled, plus the shrunk band.
    {
        TileGeom tg;
        tg.twL = tw;
        tg.thL = th;
        FftClass tf = fc[0];
        tf.tileFirst = 0;
        tf.ntiles = 1;
        NA_CUDA(launch_fwd_rows(d_tpl, tstride, step, cn, nullptr, tg, tf, ts[0], cn, st));
        MemberSet none;
        memset(&none, 0, sizeof none);
        const float scale = 1.0f / (float(p.dftW) * float(p.dftH));
        NA_CUDA(launch_cols(0, ts[0], ts[0], cn, tg, tf, 0, cn, nullptr, scale, none, 1, st));
        if (nclass == 2) NA_CUDA(launch_shrink_gather(ts[0], p.dftH, ts[1], dh2, tf.hwp, cn, st));
    }
    MemberSet ms;
    memset(&ms, 0, sizeof ms);
    ms.solo.tspec[0] = ts[0];
    ms.solo.tspec[1] = ts[1];
    ms.solo.tw = tw;
    ms.solo.th = th;
    ms.solo.rw = rw;
    ms.solo.rh = rh;
    ms.solo.roiX1 = rw;
    ms.solo.roiY1 = rh;
    ms.params = P;
    ms.map = d_map;
    ms.corr = corr;
    for (int c = 0; c < nclass; c++) {
        NA_CUDA(launch_fwd_rows(d_img, istride, step, cn, nullptr, g, fc[c], spec[c], cn, st));
        ms.scratch[c] = spec[c];
        NA_CUDA(launch_cols(1, spec[c], spec[c], cn, g, fc[c], c, cn, nullptr, 1.0f, ms, 1, st));
        NA_CUDA(launch_inv_rows(g, fc[c], c, cn, ms, 1, g.blockH, 0, 0, nullptr, nullptr, nullptr, st));
    }
    NA_CUDA(launch_norm(d_img, istride, step, ms, 1, ng, cn, parts, &F->normDone, d_out, st));
#undef NA_CUDA
    return CVM_OK;
}
