// cvm_kernels.cu -- sm_103a kernels of the TM_CCOEFF_NORMED path.
//
// Arithmetic contract: every float operation below is an explicitly
// rounded IEEE op (__fadd_rn/__fsub_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn,
// and the file is built with -fmad=false), grouped exactly like the
// reference's pinned sequence: the radix-4 butterfly and no-FMA complex
// multiply of radix4.go:17-32 and 80-149, the R2C untangle of
// impl.go:331-341, the conj-multiply of impl.go:376-388, the C2R combine of
// impl.go:405-413 and the normalisation tail of impl.go:816-849.  The
// schedule (which thread runs which butterfly, the storage order of
// intermediate rows) is free; the per-element op sequence is not.  The
// result is the reference's output bit for bit.
//
// Kernels:
//   k_gray            rgbToGray (cvmatch.go:222-240)
//   k_alpha_scan      alphaConst (cvmatch.go:146-168)
//   k_prep            templStats (impl.go:1063-1079) + the parent's alpha scan +
//                     the cn choice (cvmatch.go:82-85, matcher.go:103-112) and
//                     tail constants (impl.go:867-873, 1087), one launch
//   k_fwd_rows        forwardRowPair (impl.go:301-344) for every tile row pair
//   k_cols            colsR4Go forward / mulConjGo / colsR4Go inverse
//                     (radix4cols.go:111-125, impl.go:376-388)
//   k_inv_rows        inverseRowPair (impl.go:394-444) + channel accumulation
//   k_norm            sliding column sums (colBuildGo/colSlideGo, impl.go:708-805),
//                     normOne (impl.go:825-849), first-occurrence extrema merged
//                     in raster order (impl.go:1104-1112) by each member's last CTA
//   k_shrink_gather   shrinkInto (impl.go:591-610)
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <climits>
#include <cstdint>

#include <mutex>
#include <string>
#include <vector>

#include <algorithm>
#include <cstring>

#include "cvm_device.cuh"

namespace cvm {

// ------------------------------------------------------------ profiler
// Optional per-kernel timing: when enabled, every launch is bracketed by a
// pair of events recorded on its own stream; reading the totals
// synchronises on the recorded events.  Off by default (no events).
namespace prof {
struct Rec {
    const char *name;
    cudaEvent_t a, b;
};
std::mutex mu;
bool on = false;
std::vector<Rec> recs;
struct Total {
    std::string name;
    double ms = 0;
    unsigned long long n = 0;
};
std::vector<Total> totals;
// every launch since enabling: start and end relative to the first launch
struct Span {
    std::string name;
    double t0, t1;
};
std::vector<Span> spans;
cudaEvent_t origin = nullptr;

int begin(const char *name, cudaStream_t st) {
    if (!on) return -1;
    Rec r{name, nullptr, nullptr};
    cudaEventCreate(&r.a);
    cudaEventCreate(&r.b);
    cudaEventRecord(r.a, st);
    std::lock_guard<std::mutex> lk(mu);
    recs.push_back(r);
    return (int)recs.size() - 1;
}

void end(int idx, cudaStream_t st) {
    if (idx < 0) return;
    std::lock_guard<std::mutex> lk(mu);
    cudaEventRecord(recs[idx].b, st);
}

void collect() {
    std::lock_guard<std::mutex> lk(mu);
    for (Rec &r : recs) {
        cudaEventSynchronize(r.b);
        float ms = 0;
        cudaEventElapsedTime(&ms, r.a, r.b);
        if (!origin) {
            origin = r.a;  // kept as the timeline's zero
        }
        float t0 = 0;
        cudaEventElapsedTime(&t0, origin, r.a);
        spans.push_back(Span{r.name, t0, (double)t0 + ms});
        if (r.a != origin) cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
        Total *t = nullptr;
        for (Total &x : totals)
            if (x.name == r.name) t = &x;
        if (!t) {
            totals.push_back(Total{r.name, 0, 0});
            t = &totals.back();
        }
        t->ms += ms;
        t->n += 1;
    }
    recs.clear();
}
}  // namespace prof


namespace {


// ------------------------------------------------- radix-4 cascade passes
// The reference cascade (fftR4Scalar, radix4.go:106-149) on bit-reversed
// input: an optional radix-2 head (odd log2 n), then radix-4 stages with
// quarter sizes h = h0, 4h0, 16h0, ...  A butterfly of stage h touches
// elements base+j+{0,h,2h,3h} of a 4h-block, so the 16 elements
// B+j+h*i (i < 16, B a multiple of 16h, j < h) hold four complete
// butterflies of stage h and four of stage 4h: a thread runs two stages in
// registers per pass and the data crosses shared memory once per pass
// instead of once per stage.  Every butterfly is the same single-rounded
// op sequence with the same twiddle, so results are bit-identical to the
// stage-by-stage cascade.  Passes over one line:
//   odd log2 n:  [R2 + R4(h=2) on 8 contiguous]  then pairs from h=8
//   even log2 n: pairs from h=1
//   a trailing single radix-4 stage when one remains.

template <bool INV, typename Addr>
__device__ __forceinline__ void unit_r16(float2 *s, const Addr &addr, int base, int h, const float2 *__restrict__ tA,
                                         const float2 *__restrict__ tB) {
    float2 e[16];
#pragma unroll
    for (int i = 0; i < 16; i++) e[i] = s[addr(base + h * i)];
    const int j = base & (h - 1);
    const float2 a1 = __ldg(tA + j), a2 = __ldg(tA + h + j), a3 = __ldg(tA + 2 * h + j);
#pragma unroll
    for (int b = 0; b < 4; b++) bfly4<INV>(&e[4 * b], &e[4 * b + 1], &e[4 * b + 2], &e[4 * b + 3], a1, a2, a3);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int jj = j + h * q;
        bfly4<INV>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + jj), __ldg(tB + 4 * h + jj),
                   __ldg(tB + 8 * h + jj));
    }
#pragma unroll
    for (int i = 0; i < 16; i++) s[addr(base + h * i)] = e[i];
}

template <bool INV, typename Addr>
__device__ __forceinline__ void unit_r4(float2 *s, const Addr &addr, int base, int h, const float2 *__restrict__ t) {
    float2 e[4];
#pragma unroll
    for (int i = 0; i < 4; i++) e[i] = s[addr(base + h * i)];
    const int j = base & (h - 1);
    bfly4<INV>(&e[0], &e[1], &e[2], &e[3], __ldg(t + j), __ldg(t + h + j), __ldg(t + 2 * h + j));
#pragma unroll
    for (int i = 0; i < 4; i++) s[addr(base + h * i)] = e[i];
}

// The radix-2 head plus the h=2 radix-4 stage on 8 contiguous elements.
template <bool INV, typename Addr>
__device__ __forceinline__ void unit_head8(float2 *s, const Addr &addr, int base, const float2 *__restrict__ t) {
    float2 e[8];
#pragma unroll
    for (int i = 0; i < 8; i++) e[i] = s[addr(base + i)];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const float2 u = e[i], v = e[i + 1];
        e[i] = make_float2(__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y));
        e[i + 1] = make_float2(__fsub_rn(u.x, v.x), __fsub_rn(u.y, v.y));
    }
#pragma unroll
    for (int j = 0; j < 2; j++)
        bfly4<INV>(&e[j], &e[j + 2], &e[j + 4], &e[j + 6], __ldg(t + j), __ldg(t + 2 + j), __ldg(t + 4 + j));
#pragma unroll
    for (int i = 0; i < 8; i++) s[addr(base + i)] = e[i];
}

// The radix-2 head alone (n = 2, 4-point odd... only n == 2 needs it).
template <typename Addr>
__device__ __forceinline__ void unit_r2(float2 *s, const Addr &addr, int base) {
    const float2 u = s[addr(base)], v = s[addr(base + 1)];
    s[addr(base)] = make_float2(__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y));
    s[addr(base + 1)] = make_float2(__fsub_rn(u.x, v.x), __fsub_rn(u.y, v.y));
}

// Runs the whole cascade over `lines` independent transforms of length n
// (log2n), element (line, i) at s[la(line, i)].  LINE_FAST maps consecutive
// threads to consecutive lines (column strips, lines a power of two);
// otherwise to consecutive units of one line (row lines).  Ends with a
// barrier.
template <bool INV, bool LINE_FAST = false, typename LineAddr>
__device__ void fft_cascade(float2 *s, int n, int log2n, int lines, const LineAddr &la,
                            const float2 *__restrict__ tri) {
    const int tid = threadIdx.x, nt = blockDim.x;
    int h = 1;
    const float2 *t = tri;
    if (log2n & 1) {
        if (n == 2) {
            for (int u = tid; u < lines; u += nt) {
                auto addr = [&](int i) { return la(u, i); };
                unit_r2(s, addr, 0);
            }
            __syncthreads();
            return;
        }
        const int units = n >> 3;
        for (int u = tid; u < lines * units; u += nt) {
            const int line = LINE_FAST ? (u & (lines - 1)) : u / units;
            const int base = (LINE_FAST ? (u / lines) : (u - line * units)) << 3;
            auto addr = [&](int i) { return la(line, i); };
            unit_head8<INV>(s, addr, base, t);
        }
        __syncthreads();
        t += 6;  // the h=2 stage's table
        h = 8;
    }
    while (16 * h <= n) {
        const int units = n >> 4;
        const float2 *tB = t + 3 * h;
        for (int u = tid; u < lines * units; u += nt) {
            const int line = LINE_FAST ? (u & (lines - 1)) : u / units;
            const int v = LINE_FAST ? u / lines : u - line * units;
            const int j = v & (h - 1), blk = v >> (31 - __clz(h));
            const int base = blk * 16 * h + j;
            auto addr = [&](int i) { return la(line, i); };
            unit_r16<INV>(s, addr, base, h, t, tB);
        }
        __syncthreads();
        t = tB + 12 * h;
        h *= 16;
    }
    if (4 * h <= n) {
        const int units = n >> 2;
        for (int u = tid; u < lines * units; u += nt) {
            const int line = LINE_FAST ? (u & (lines - 1)) : u / units;
            const int v = LINE_FAST ? u / lines : u - line * units;
            const int j = v & (h - 1), blk = v >> (31 - __clz(h));
            const int base = blk * 4 * h + j;
            auto addr = [&](int i) { return la(line, i); };
            unit_r4<INV>(s, addr, base, h, t);
        }
        __syncthreads();
    }
}


// The column twin (colsR4Go, radix4cols.go:35-125) on a [n x SC] strip in
// shared memory, element (row r, column c) at s[r*SC + c]; RMAP conjugates
// every row access by the bit reversal (the inverse path's rmap = brev).
template <bool INV, bool RMAP>
__device__ void fft_cols(float2 *s, int n, int log2n, int SC, int logSC, const float2 *__restrict__ tri) {
    auto la = [=](int c, int r) {
        const int rr = RMAP ? brev_bits(r, log2n) : r;
        return (rr << logSC) + c;
    };
    fft_cascade<INV, true>(s, n, log2n, SC, la, tri);
}


// ------------------------------------------------------------ gray/alpha

__global__ void k_gray(const uint8_t *__restrict__ src, long long sstride, int w, int h,
                       uint8_t *__restrict__ dst, long long dstride) {
    const int y = blockIdx.y;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < w; x += gridDim.x * blockDim.x) {
        const uint8_t *p = src + (long long)y * sstride + 4LL * x;
        const uint32_t r = p[0], g = p[1], b = p[2];
        dst[(long long)y * dstride + x] = (uint8_t)((4899u * r + 9617u * g + 1868u * b + 8192u) >> 14);
    }
}

__global__ void k_alpha_scan(const uint8_t *__restrict__ img, long long stride, int w, int h,
                             unsigned int *mismatch) {
    const uint8_t a0 = img[3];
    const int y = blockIdx.y;
    bool bad = false;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < w; x += gridDim.x * blockDim.x)
        bad |= img[(long long)y * stride + 4LL * x + 3] != a0;
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(mismatch, 1u);
}

// ----------------------------------------------------- statistics + cn

// Derives the effective channel count (cvmatch.go:82-85, matcher.go:103-112)
// and the tail constants of one template with the reference's
// double-precision sequences (impl.go:867-873, 1087).  Runs once per call,
// in the last CTA of k_prep.
__device__ void finalize_params(DevParams &p, const DevFrame &F, int *cnMax) {
    int cn = p.cnFixed;
    if (p.mode == 1) cn = (p.alphaMismatch == 0 && F.alphaMismatch == 0) ? 3 : 4;
    const long long area = (long long)p.tw * p.th;
    long long vs = 0;
    for (int k = 0; k < cn; k++) {
        const long long sk = (long long)p.tsum[k];
        vs += area * (long long)p.tsq[k] - sk * sk;
    }
    p.cn = cn;
    p.varSum = vs;
    p.flat = vs == 0;
    const double ad = __dmul_rn((double)p.tw, (double)p.th);
    p.templNorm = __double2float_rn(__dsqrt_rn(__ddiv_rn(__ll2double_rn(vs), ad)));
    p.varScale = __double2float_rn(__ddiv_rn(1.0, ad));
    p.numScale = cn == 1 ? __double2float_rn(__ddiv_rn(__ll2double_rn((long long)p.tsum[0]), ad)) : p.varScale;
    if (!p.flat) atomicMax(cnMax, cn);
}

struct PrepArgs {
    const uint8_t *tpl;      // template pixels whose statistics P[0] accumulates (nullptr: cached)
    long long tstride;
    int tw, th, tstep, cnStats, tplCtas;
    const uint8_t *parent;   // parent whose alpha plane is scanned (nullptr: no scan)
    long long pstride;
    int pw, ph, parentCtas;
    int pvec16;              // parent rows 16-byte aligned: scan with vector loads
    DevParams *P;
    int n;                   // params to finalize
    int setInit;             // store mode/cnFixed/tw/th of `init` into P[0] first
    int initMode, initCnFixed;
    DevFrame *F;
};

// One launch for everything a call needs before its transforms: exact
// template sums and squared sums (templStats, impl.go:1063-1079) with the
// template's alpha-constancy flag, the parent's alpha scan (alphaConst,
// cvmatch.go:146-168), and -- in the CTA that finishes last -- the cn
// choice and tail constants of every member.  P and F are zeroed first.
__global__ void k_prep(PrepArgs a) {
    griddep_launch();  // the frame's row transform may start placing CTAs
    __shared__ int isLast;
    const int tid = threadIdx.x, nt = blockDim.x;
    bool bad = false;
    if ((int)blockIdx.x < a.tplCtas) {
        unsigned long long sm[4] = {0, 0, 0, 0}, q[4] = {0, 0, 0, 0};
        const int total = a.tw * a.th;  // below the statistics cap, < 2^31
        const uint8_t a0 = a.tstep == 4 ? a.tpl[3] : 0;
        for (int i = blockIdx.x * nt + tid; i < total; i += a.tplCtas * nt) {
            const int y = i / a.tw, x = i - y * a.tw;
            const uint8_t *p = a.tpl + (long long)y * a.tstride + (long long)x * a.tstep;
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (k < a.cnStats) {
                    const unsigned v = p[k];
                    sm[k] += v;
                    q[k] += v * v;
                }
            if (a.tstep == 4) bad |= p[3] != a0;
        }
#pragma unroll
        for (int k = 0; k < 4; k++)
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sm[k] += __shfl_down_sync(0xffffffffu, sm[k], o);
                q[k] += __shfl_down_sync(0xffffffffu, q[k], o);
            }
        // warp totals -> one set of atomics per CTA
        __shared__ unsigned long long red[kThreads / 32][8];
        __shared__ int redBad;
        if (tid == 0) redBad = 0;
        __syncthreads();
        const bool anyBad = __any_sync(0xffffffffu, bad);
        if ((tid & 31) == 0) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                red[tid >> 5][k] = sm[k];
                red[tid >> 5][4 + k] = q[k];
            }
            if (anyBad) redBad = 1;
        }
        __syncthreads();
        if (tid < 8) {
            unsigned long long t = 0;
            for (int w = 0; w < (nt >> 5); w++) t += red[w][tid];
            const int k = tid & 3;
            if (k < a.cnStats && t) atomicAdd(tid < 4 ? &a.P[0].tsum[k] : &a.P[0].tsq[k], t);
        }
        if (tid == 0 && redBad) atomicOr(&a.P[0].alphaMismatch, 1u);
    } else if (a.parent) {
        const int c = blockIdx.x - a.tplCtas;
        const uint8_t a0 = a.parent[3];
        if (a.pvec16) {
            // four pixels per 16-byte load, the loads of several items in flight
            const unsigned int want = (unsigned int)a0 << 24;
            const int nv = a.pw >> 2, items = a.ph * nv, stride = a.parentCtas * nt;
            unsigned int acc = 0u;
            for (int it0 = c * nt + tid; it0 < items; it0 += 8 * stride) {
                uint4 w[8];
#pragma unroll
                for (int k = 0; k < 8; k++) {  // eight loads in flight
                    const int it = it0 + k * stride;
                    w[k] = make_uint4(want, want, want, want);
                    if (it < items) {
                        const int y = it / nv, v = it - y * nv;
                        w[k] = __ldg(reinterpret_cast<const uint4 *>(a.parent + (long long)y * a.pstride) + v);
                    }
                }
#pragma unroll
                for (int k = 0; k < 8; k++)
                    acc |= ((w[k].x ^ want) | (w[k].y ^ want) | (w[k].z ^ want) | (w[k].w ^ want)) & 0xff000000u;
            }
            bad = acc != 0u;
            // the last pw % 4 pixels of every row
            for (int y = c * nt + tid; y < a.ph * (a.pw & 3); y += a.parentCtas * nt) {
                const int r = y / (a.pw & 3), x = 4 * nv + (y - r * (a.pw & 3));
                bad |= a.parent[(long long)r * a.pstride + 4LL * x + 3] != a0;
            }
        } else {
            for (int y = c; y < a.ph; y += a.parentCtas) {
                const uint8_t *row = a.parent + (long long)y * a.pstride + 3;
                for (int x = tid; x < a.pw; x += nt) bad |= row[4LL * x] != a0;
            }
        }
        if (__any_sync(0xffffffffu, bad) && (tid & 31) == 0) atomicOr(&a.F->alphaMismatch, 1u);
    }
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        isLast = atomicAdd(&a.F->done, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (!isLast) return;
    __threadfence();
    if (tid == 0 && a.setInit) {
        a.P[0].mode = a.initMode;
        a.P[0].cnFixed = a.initCnFixed;
        a.P[0].tw = a.tw;
        a.P[0].th = a.th;
    }
    __syncthreads();
    DevFrame F;
    F.alphaMismatch = ((volatile DevFrame *)a.F)->alphaMismatch;
    for (int i = tid; i < a.n; i += nt) {
        DevParams p;
        const volatile DevParams *src = a.P + i;
        for (int k = 0; k < 4; k++) {
            p.tsum[k] = src->tsum[k];
            p.tsq[k] = src->tsq[k];
        }
        p.alphaMismatch = src->alphaMismatch;
        p.mode = src->mode;
        p.cnFixed = src->cnFixed;
        p.tw = src->tw;
        p.th = src->th;
        finalize_params(p, F, &a.F->cnMax);
        a.P[i] = p;
    }
}

// --------------------------------------------------------- forward rows

// forwardRowPair (impl.go:301-344) for P row pairs x C channels of one
// tile: pack two image rows into one complex row, transform, untangle into
// the two real-row spectra at their bit-reversed column-FFT slots.
__global__ void k_fwd_rows(const uint8_t *__restrict__ img, long long istride, int step,
                           int chanCount, const int *cnDev, int chanFirst, int chanGroup, TileGeom g,
                           FftClass fc, float2 *__restrict__ spec, int cnS, int pairsPerCta) {
    extern __shared__ float2 smem[];
    const int tile = fc.tileFirst + blockIdx.y;
    const TileBox b = tile_box(g, tile);
    const int nrows = min(b.loadH, fc.dftH);
    const int pair0 = blockIdx.x * pairsPerCta;
    if (2 * pair0 >= nrows) return;
    const int cnEff = cnDev ? min(*cnDev, chanCount) : chanCount;
    const int cn = min(cnEff - chanFirst, chanGroup);  // channels of this launch's group
    if (cn <= 0) return;
    const int P = min(pairsPerCta, (nrows - 2 * pair0 + 1) >> 1);
    const int lines = P * cn;
    const int n = fc.n, log2n = fc.log2n, ld = padded_len(n);
    const int tid = threadIdx.x, nt = blockDim.x;
    const long long rowBase = (long long)b.y0 * istride + (long long)b.x0 * step;
    for (int line = 0; line < lines; line++) {
        const int p = line / cn, k = chanFirst + line - p * cn;
        const int r = 2 * (pair0 + p);
        const bool two = r + 1 < b.loadH;
        const uint8_t *pa = img + rowBase + (long long)r * istride + k;
        float2 *dl = smem + line * ld;
        for (int x = tid; x < n; x += nt) {
            float2 v = make_float2(0.f, 0.f);
            if (x < b.loadW) {
                const uint8_t *q = pa + (long long)x * step;
                v.x = (float)q[0];
                if (two) v.y = (float)q[istride];
            }
            dl[padi(brev_bits(x, log2n))] = v;
        }
    }
    __syncthreads();
    auto la = [=](int line, int i) { return line * ld + padi(i); };
    fft_cascade<false>(smem, n, log2n, lines, la, fc.triW);
    const int hw = fc.hw, mask = n - 1;
    const size_t chanStride = (size_t)fc.dftH * fc.hwp;
    float2 *tbase = spec + (size_t)(tile - fc.tileFirst) * cnS * chanStride;
    for (int line = 0; line < lines; line++) {
        const int p = line / cn, k = chanFirst + line - p * cn;
        const int r = 2 * (pair0 + p);
        const float2 *zl = smem + line * ld;
        float2 *cb = tbase + (size_t)k * chanStride;
        float2 *sa = cb + (size_t)brev_bits(r, fc.log2H) * fc.hwp;
        float2 *sb = cb + (size_t)brev_bits(r + 1, fc.log2H) * fc.hwp;
        for (int kk = tid; kk < hw; kk += nt) {
            const float2 zk = zl[padi(kk)], zn = zl[padi((n - kk) & mask)];
            sa[kk] = make_float2(__fmul_rn(0.5f, __fadd_rn(zk.x, zn.x)), __fmul_rn(0.5f, __fsub_rn(zk.y, zn.y)));
            sb[kk] = make_float2(__fmul_rn(0.5f, __fadd_rn(zk.y, zn.y)), __fmul_rn(0.5f, __fsub_rn(zn.x, zk.x)));
        }
    }
}

// --------------------------------------------------------------- columns



// Column pass over one [dftH x SC] strip of one (member, tile, channel).
__global__ void k_cols(ColsArgs a) {
    extern __shared__ float2 smem[];
    const FftClass &fc = a.fc;
    const int tileLocal = blockIdx.z % fc.ntiles;
    const int slot = blockIdx.z / fc.ntiles;
    const int tile = fc.tileFirst + tileLocal;
    const int k = blockIdx.y;
    const DevMember *m = a.mode == 0 ? nullptr : &member_of(a.ms, slot);
    const DevParams *Pm = m ? a.ms.params + m->pIdx : nullptr;
    int cn;
    if (m)
        cn = Pm->cn;
    else
        cn = a.cnDev ? min(*a.cnDev, a.chanCount) : a.chanCount;
    if (k >= cn) return;
    if (Pm && Pm->flat) return;
    const int SC = a.SC, logSC = a.logSC;
    const int c0 = blockIdx.x * SC;
    const int H = fc.dftH, log2H = fc.log2H, hwp = fc.hwp;
    const int wv = min(SC, fc.hw - c0);
    const size_t chanStride = (size_t)H * hwp;
    const TileBox b = tile_box(a.g, tile);
    if (m && a.ms.anyRoi && roi_misses_tile(a.g, tile, b, *m)) return;  // outside the member's ROI
    const int tid = threadIdx.x, nt = blockDim.x;

    const float2 *src = a.in + ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
    if (a.mode == 2) {
        // Natural-order forward spectrum of the frame tile.
        for (int idx = tid; idx < (H << logSC); idx += nt) {
            const int r = idx >> logSC, c = idx & (SC - 1);
            smem[idx] = c < wv ? src[(size_t)r * hwp + c] : make_float2(0.f, 0.f);
        }
    } else {
        // Forward-rows output: logical row brev(s) sits at slot s; rows at or
        // past `loaded` were never written and are zero (impl.go:352-356).
        const int loaded = min(H, (b.loadH + 1) & ~1);
        for (int idx = tid; idx < (H << logSC); idx += nt) {
            const int s = idx >> logSC, c = idx & (SC - 1);
            float2 v = make_float2(0.f, 0.f);
            if (c < wv && brev_bits(s, log2H) < loaded) v = src[(size_t)s * hwp + c];
            smem[idx] = v;
        }
    }
    __syncthreads();
    if (a.mode != 2) fft_cols<false, false>(smem, H, log2H, SC, logSC, fc.triH);
    if (a.mode == 0) {
        float2 *dst = a.out + ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
        const float sc = a.scale;
        for (int idx = tid; idx < (H << logSC); idx += nt) {
            const int r = idx >> logSC, c = idx & (SC - 1);
            if (c < wv) {
                float2 v = smem[idx];
                if (sc != 1.0f) v = make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
                dst[(size_t)r * hwp + c] = v;
            }
        }
        return;
    }
    // spec *= conj(tspec) (mulConjGo, impl.go:376-388), natural order.
    const float2 *ts = m->tspec[a.cls] + (size_t)k * chanStride + c0;
    for (int idx = tid; idx < (H << logSC); idx += nt) {
        const int r = idx >> logSC, c = idx & (SC - 1);
        if (c < wv) {
            const float2 av = smem[idx], bv = __ldg(ts + (size_t)r * hwp + c);
            const float re = __fadd_rn(__fmul_rn(av.x, bv.x), __fmul_rn(av.y, bv.y));
            const float im = __fsub_rn(__fmul_rn(av.y, bv.x), __fmul_rn(av.x, bv.y));
            smem[idx] = make_float2(re, im);
        }
    }
    __syncthreads();
    fft_cols<true, true>(smem, H, log2H, SC, logSC, fc.triH);
    // Spatial row y now sits at slot brev(y); the inverse rows read rows
    // y < bh (rounded up to the row pair).
    const int ty = tile / a.g.ntx;
    const int bh = (ty == a.g.nty - 1) ? m->rh - b.y0 : a.g.blockH;
    const int rowsOut = min(H, (bh + 1) & ~1);
    float2 *dst = a.ms.scratch[a.cls] + (size_t)slot * a.ms.scratchStride[a.cls] +
                  ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
    for (int idx = tid; idx < (H << logSC); idx += nt) {
        const int s = idx >> logSC, c = idx & (SC - 1);
        if (c < wv && brev_bits(s, log2H) < rowsOut) dst[(size_t)s * hwp + c] = smem[idx];
    }
}

// ------------------------------------------- column pass, even log2 dftH
// With the reference's storage relabelling (forward rows stored at
// bit-reversed slots, inverse read through rmap = brev), the forward
// cascade's last pass and the inverse cascade's first pass act on the same
// element sets when log2 dftH is even: the 16 rows {B + S*c} (S = dftH/16)
// hold complete butterflies of the forward's last stage(s), and through the
// bit reversal the same rows are one contiguous 16-slot block of the
// inverse's first two stages (slot 16a+r <-> row B + S*brev4(r)).  So the
// forward's last pass, the conj-multiply and the inverse's first pass run
// in registers in one sweep; the forward's first pass reads global memory
// directly and the inverse's last pass writes it.  Every butterfly keeps
// the reference's op sequence and twiddle.

template <bool INV, typename LD, typename ST>
__device__ __forceinline__ void unit_r16_io(const LD &ld, const ST &st, int base, int h,
                                            const float2 *__restrict__ tA, const float2 *__restrict__ tB) {
    float2 e[16];
#pragma unroll
    for (int i = 0; i < 16; i++) e[i] = ld(base + h * i);
    const int j = base & (h - 1);
    const float2 a1 = __ldg(tA + j), a2 = __ldg(tA + h + j), a3 = __ldg(tA + 2 * h + j);
#pragma unroll
    for (int b = 0; b < 4; b++) bfly4<INV>(&e[4 * b], &e[4 * b + 1], &e[4 * b + 2], &e[4 * b + 3], a1, a2, a3);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int jj = j + h * q;
        bfly4<INV>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + jj), __ldg(tB + 4 * h + jj),
                   __ldg(tB + 8 * h + jj));
    }
#pragma unroll
    for (int i = 0; i < 16; i++) st(base + h * i, e[i]);
}

template <bool INV, typename LD, typename ST>
__device__ __forceinline__ void unit_r4_io(const LD &ld, const ST &st, int base, int h, const float2 *__restrict__ t) {
    float2 e[4];
#pragma unroll
    for (int i = 0; i < 4; i++) e[i] = ld(base + h * i);
    const int j = base & (h - 1);
    bfly4<INV>(&e[0], &e[1], &e[2], &e[3], __ldg(t + j), __ldg(t + h + j), __ldg(t + 2 * h + j));
#pragma unroll
    for (int i = 0; i < 4; i++) st(base + h * i, e[i]);
}

__device__ __forceinline__ int brev4c(int r) { return ((r & 1) << 3) | ((r & 2) << 1) | ((r & 4) >> 1) | ((r & 8) >> 3); }

// One even-log2 radix pass (r16 at quarter h, or r4 at h) over all columns
// of the strip with the given element I/O.  Ends with a barrier.
template <bool INV, typename LD, typename ST>
__device__ __forceinline__ void even_pass(int H, int SC, int logSC, bool r16, int h, const float2 *t, const LD &ld,
                                          const ST &st) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int units = r16 ? H >> 4 : H >> 2;
    const int lh = 31 - __clz(h);
    for (int u = tid; u < (units << logSC); u += nt) {
        const int c = u & (SC - 1), v = u >> logSC;
        const int j = v & (h - 1), blk = v >> lh;
        auto l = [&](int i) { return ld(c, i); };
        auto w = [&](int i, float2 x) { st(c, i, x); };
        if (r16)
            unit_r16_io<INV>(l, w, blk * 16 * h + j, h, t, t + 3 * h);
        else
            unit_r4_io<INV>(l, w, blk * 4 * h + j, h, t);
    }
    __syncthreads();
}

// The middle sweep over the row sets {B + S*c : c < M} (M = 16, or 4 when
// dftH = 4): forward's last pass (r16 at quarter hL, or the trailing r4 at
// hL = 4S), conj-multiply, inverse's first pass; the results go to shared
// memory (or straight to global memory when the transform has one pass).
template <int M, int MODE, typename LDX, typename STI, typename STS>
__device__ __forceinline__ void middle_sweep(int S, int logSC, int SC, int L, bool fwdLastR16, int hL,
                                             const float2 *__restrict__ tri, const float2 *__restrict__ ts, int hwp,
                                             int wv, const LDX &ldx, const STI &store_inv, const STS &store_smem,
                                             bool onlyPass) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const float2 zero = make_float2(0.f, 0.f);
    const float2 *tL = tri + (hL - 1);
    for (int u = tid; u < (S << logSC); u += nt) {
        const int c = u & (SC - 1), B = u >> logSC;
        float2 x[M];
#pragma unroll
        for (int ci = 0; ci < M; ci++) x[ci] = ldx(c, B + S * ci);
        if (MODE == 1) {
            if (M == 16 && fwdLastR16) {
                const float2 a1 = __ldg(tL + B), a2 = __ldg(tL + hL + B), a3 = __ldg(tL + 2 * hL + B);
#pragma unroll
                for (int q = 0; q < M / 4; q++)
                    bfly4<false>(&x[4 * q], &x[4 * q + 1], &x[4 * q + 2], &x[4 * q + 3], a1, a2, a3);
                const float2 *tB = tL + 3 * hL;
#pragma unroll
                for (int q = 0; q < M / 4; q++) {
                    const int jj = B + hL * q;
                    bfly4<false>(&x[q], &x[q + M / 4], &x[q + M / 2], &x[q + 3 * M / 4], __ldg(tB + jj),
                                 __ldg(tB + 4 * hL + jj), __ldg(tB + 8 * hL + jj));
                }
            } else {
                // trailing r4 stage hL = 4S (or dftH = 4): butterflies j = B + S*q
#pragma unroll
                for (int q = 0; q < M / 4; q++) {
                    const int j = B + S * q;
                    bfly4<false>(&x[q], &x[q + M / 4], &x[q + M / 2], &x[q + 3 * M / 4], __ldg(tL + j),
                                 __ldg(tL + hL + j), __ldg(tL + 2 * hL + j));
                }
            }
        }
        // spec *= conj(tspec) (mulConjGo, impl.go:376-388)
#pragma unroll
        for (int ci = 0; ci < M; ci++) {
            const float2 av = x[ci], bv = c < wv ? __ldg(ts + (size_t)(B + S * ci) * hwp + c) : zero;
            x[ci] = make_float2(__fadd_rn(__fmul_rn(av.x, bv.x), __fmul_rn(av.y, bv.y)),
                                __fsub_rn(__fmul_rn(av.y, bv.x), __fmul_rn(av.x, bv.y)));
        }
        // inverse's first pass: logical slot base+r holds row B + S*brev(r)
        const int abase = brev_bits(B, L);
        float2 e[M];
#pragma unroll
        for (int r = 0; r < M; r++) e[r] = x[M == 16 ? brev4c(r) : ((r & 1) << 1) | ((r & 2) >> 1)];
        const float2 a1 = __ldg(tri), a2 = __ldg(tri + 1), a3 = __ldg(tri + 2);
#pragma unroll
        for (int q = 0; q < M / 4; q++) bfly4<true>(&e[4 * q], &e[4 * q + 1], &e[4 * q + 2], &e[4 * q + 3], a1, a2, a3);
        if (M == 16) {
            const float2 *tB = tri + 3;
#pragma unroll
            for (int q = 0; q < 4; q++)
                bfly4<true>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + q), __ldg(tB + 4 + q), __ldg(tB + 8 + q));
        }
#pragma unroll
        for (int r = 0; r < M; r++) {
            const int row = B + S * (M == 16 ? brev4c(r) : (((r & 1) << 1) | ((r & 2) >> 1)));
            if (onlyPass)
                store_inv(c, abase + r, e[r]);
            else
                store_smem(c, row, e[r]);
        }
    }
    __syncthreads();
}

template <int MODE>
__global__ void __launch_bounds__(256, 3) k_cols_even(ColsArgs a) {
    extern __shared__ float2 smem[];
    const FftClass &fc = a.fc;
    const int tileLocal = blockIdx.z % fc.ntiles;
    const int slot = blockIdx.z / fc.ntiles;
    const int tile = fc.tileFirst + tileLocal;
    const int k = blockIdx.y;
    const DevMember *m = MODE == 0 ? nullptr : &member_of(a.ms, slot);
    const DevParams *Pm = m ? a.ms.params + m->pIdx : nullptr;
    int cn;
    if (m)
        cn = Pm->cn;
    else
        cn = a.cnDev ? min(*a.cnDev, a.chanCount) : a.chanCount;
    if (k >= cn) return;
    if (Pm && Pm->flat) return;
    const int SC = a.SC, logSC = a.logSC;
    const int c0 = blockIdx.x * SC;
    const int H = fc.dftH, L = fc.log2H, hwp = fc.hwp;
    const int wv = min(SC, fc.hw - c0);
    const size_t chanStride = (size_t)H * hwp;
    const TileBox b = tile_box(a.g, tile);
    if (m && a.ms.anyRoi && roi_misses_tile(a.g, tile, b, *m)) return;  // outside the member's ROI
    const float2 *tri = fc.triH;
    const float2 zero = make_float2(0.f, 0.f);
    // even-log2 passes: r16 at h = 16^p for p < L/4, then r4 at h = 16^(L/4)
    // when L % 4 == 2; stage h's twiddles start at tri + h - 1
    const int nR16 = L >> 2;
    const int nPass = nR16 + ((L & 2) ? 1 : 0);
    auto passH = [](int p) { return 1 << (4 * p); };
    auto passR16 = [=](int p) { return p < nR16; };
    const float2 *src = a.in + ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
    const int loaded = min(H, (b.loadH + 1) & ~1);
    auto gload_slots = [=](int c, int s) -> float2 {  // forward-rows output at slot s
        return (c < wv && brev_bits(s, L) < loaded) ? src[(size_t)s * hwp + c] : zero;
    };
    auto sld = [=](int c, int i) { return smem[(i << logSC) + c]; };
    auto sst = [=](int c, int i, float2 v) { smem[(i << logSC) + c] = v; };
    auto sld_r = [=](int c, int i) { return smem[(brev_bits(i, L) << logSC) + c]; };
    auto sst_r = [=](int c, int i, float2 v) { smem[(brev_bits(i, L) << logSC) + c] = v; };

    if (MODE == 0) {
        float2 *dst = a.out + ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
        const float sc = a.scale;
        auto gst_nat = [=](int c, int i, float2 v) {
            if (c < wv) {
                if (sc != 1.0f) v = make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
                dst[(size_t)i * hwp + c] = v;
            }
        };
        for (int p = 0; p < nPass; p++) {
            const int h = passH(p);
            const float2 *t = tri + (h - 1);
            const bool first = p == 0, last = p == nPass - 1;
            if (first && last)
                even_pass<false>(H, SC, logSC, passR16(p), h, t, gload_slots, gst_nat);
            else if (first)
                even_pass<false>(H, SC, logSC, passR16(p), h, t, gload_slots, sst);
            else if (last)
                even_pass<false>(H, SC, logSC, passR16(p), h, t, sld, gst_nat);
            else
                even_pass<false>(H, SC, logSC, passR16(p), h, t, sld, sst);
        }
        return;
    }
    if (MODE == 1)
        for (int p = 0; p + 1 < nPass; p++) {
            const int h = passH(p);
            if (p == 0)
                even_pass<false>(H, SC, logSC, passR16(p), h, tri + (h - 1), gload_slots, sst);
            else
                even_pass<false>(H, SC, logSC, passR16(p), h, tri + (h - 1), sld, sst);
        }
    const int ty = tile / a.g.ntx;
    const int bh = (ty == a.g.nty - 1) ? m->rh - b.y0 : a.g.blockH;
    const int rowsOut = min(H, (bh + 1) & ~1);
    float2 *dst = a.ms.scratch[a.cls] + (size_t)slot * a.ms.scratchStride[a.cls] +
                  ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
    auto gst_inv = [=](int c, int i, float2 v) {  // logical slot i -> row brev(i)
        if (c < wv && i < rowsOut) dst[(size_t)brev_bits(i, L) * hwp + c] = v;
    };
    const float2 *ts = m->tspec[a.cls] + (size_t)k * chanStride + c0;
    const bool onlyPass = nPass == 1;
    const int hL = passH(nPass - 1);
    const bool fwdLastR16 = passR16(nPass - 1);
    auto ld_mode2 = [=](int c, int row) { return c < wv ? src[(size_t)row * hwp + c] : zero; };
    auto ld_mid = [=](int c, int row) { return onlyPass ? gload_slots(c, row) : smem[(row << logSC) + c]; };
    if (H >= 16) {
        const int S = H >> 4;
        if (MODE == 2)
            middle_sweep<16, 2>(S, logSC, SC, L, fwdLastR16, hL, tri, ts, hwp, wv, ld_mode2, gst_inv, sst, onlyPass);
        else
            middle_sweep<16, 1>(S, logSC, SC, L, fwdLastR16, hL, tri, ts, hwp, wv, ld_mid, gst_inv, sst, onlyPass);
    } else {
        if (MODE == 2)
            middle_sweep<4, 2>(1, logSC, SC, L, false, 1, tri, ts, hwp, wv, ld_mode2, gst_inv, sst, onlyPass);
        else
            middle_sweep<4, 1>(1, logSC, SC, L, false, 1, tri, ts, hwp, wv, ld_mid, gst_inv, sst, onlyPass);
    }
    for (int p = 1; p < nPass; p++) {
        const int h = passH(p);
        if (p == nPass - 1)
            even_pass<true>(H, SC, logSC, passR16(p), h, tri + (h - 1), sld_r, gst_inv);
        else
            even_pass<true>(H, SC, logSC, passR16(p), h, tri + (h - 1), sld_r, sst_r);
    }
}

// ------------------------------------------------------- inverse rows

// Round-to-nearest-even of a positive integer to `bits` significant bits.
__device__ __forceinline__ unsigned long long rn_bits(unsigned long long a, int bits) {
    const int bl = 64 - __clzll((long long)a);
    if (bl <= bits) return a;
    const int sh = bl - bits;
    unsigned long long q = a >> sh;
    const unsigned long long rem = a & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (q & 1ull))) q++;
    return q << sh;
}

// Correctly rounded float32 of an unsigned 64-bit integer without the 64-bit
// conversion instruction (it runs on the FP64 pipe, which GB300 provisions
// at a small fraction of FP32): the top 32 bits with the OR of the dropped
// bits as a sticky bit round exactly like the full value under one
// u32->f32 rounding, and the exponent is then adjusted exactly.
__device__ __forceinline__ float u64_to_f32_rn(unsigned long long a) {
    const unsigned int hi = (unsigned int)(a >> 32), lo = (unsigned int)a;
    if (hi == 0) return __uint2float_rn(lo);
    const int sh = 32 - __clz(hi);  // bits above the low word, 1..32
    const unsigned int t = (unsigned int)(a >> sh);
    const unsigned int dropped = sh == 32 ? lo : (lo & ((1u << sh) - 1u));
    const float f = __uint2float_rn(t | (dropped != 0u));
    return __int_as_float(__float_as_int(f) + (sh << 23));
}

// float32(float64(v)) (impl.go:902-1009): the conversion to float64 rounds
// to 53 bits, the one to float32 to 24 bits, both to nearest even.  Below
// 2^53 the first rounding is exact, so a single rounding gives the bits.
__device__ __forceinline__ float f32_via_f64(long long v) {
    unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    if (a >= (1ull << 53)) a = rn_bits(a, 53);
    const float f = u64_to_f32_rn(a);
    return v < 0 ? -f : f;
}

// normOne (impl.go:825-849).  s2 is the exact integer: lim = min(eps *
// float32(s2), 0.5) is 0.5 for every s2 >= 2^19 (eps * 2^19 = 0.625), so
// the conversion is only needed below 2^24, where it is exact.
__device__ __forceinline__ float norm_one(float num, float lane0, float idiff, unsigned long long s2i,
                                          float numScale, float varScale, float templNorm) {
    const float eps = 1.1920928955078125e-06f;  // 10 * 2^-23, exact in float32
    num = __fsub_rn(num, __fmul_rn(lane0, numScale));
    const float diff2 = __fmul_rn(idiff, varScale);
    float lim = 0.5f;
    if (s2i < (1ull << 24)) {
        lim = __fmul_rn(eps, __uint2float_rn((unsigned int)s2i));
        if (lim > 0.5f) lim = 0.5f;
    }
    float den = 0.f;
    if (diff2 > lim) den = __fmul_rn(__fsqrt_rn(diff2), templNorm);
    const float an = fabsf(num);
    if (an < den) return __fdiv_rn(num, den);
    if (an < __fmul_rn(den, 1.125f)) return num > 0.f ? 1.f : -1.f;
    return 0.f;
}



// inverseRowPair (impl.go:394-444) for P row pairs of one (member, tile):
// combine, inverse row transform, the channels accumulated in channel order
// (the add=k>0 emit of impl.go:425-443), then the rest of normOne
// (impl.go:825-849) with the per-result (t, den) the statistics kernel
// prepared, first-occurrence extrema per CTA, and the member's last CTA
// merges them in raster-order semantics (impl.go:1104-1112).
__global__ void __launch_bounds__(256, 3) k_inv_rows(InvArgs a) {
    extern __shared__ float2 smem[];
    __shared__ Ext shExt[kThreads / 32];
    __shared__ int isLast;
    const FftClass &fc = a.fc;
    const int tileLocal = blockIdx.y;
    const int tile = fc.tileFirst + tileLocal;
    const int slot = blockIdx.z;
    const DevMember &m = member_of(a.ms, slot);
    const DevParams &Pm = a.ms.params[m.pIdx];
    const TileBox tb = tile_box(a.g, tile);
    const int tx = tile % a.g.ntx, ty = tile / a.g.ntx;
    const int bw = (tx == a.g.ntx - 1) ? m.rw - tb.x0 : a.g.blockW;
    const int bh = (ty == a.g.nty - 1) ? m.rh - tb.y0 : a.g.blockH;
    const int pair0 = blockIdx.x * a.pairsPerCta;
    // the CTA's row pairs; none when its results all lie outside the
    // member's region of interest (no transform, no extrema)
    int P = 2 * pair0 < bh ? min(a.pairsPerCta, (bh - 2 * pair0 + 1) >> 1) : 0;
    if (P > 0 && a.ms.anyRoi) {
        const int ya = tb.y0 + 2 * pair0, yb = tb.y0 + min(2 * (pair0 + P), bh);
        if (ya >= m.roiY1 || yb <= m.roiY0 || tb.x0 >= m.roiX1 || tb.x0 + bw <= m.roiX0) P = 0;
    }
    const int n = fc.n, log2n = fc.log2n, hw = fc.hw, hwp = fc.hwp, ld = padded_len(n);
    const int tid = threadIdx.x, nt = blockDim.x;
    const bool flat = Pm.flat != 0;
    float *acc = reinterpret_cast<float *>(smem + (size_t)a.pairsPerCta * ld);  // [P][2][n]
    Ext e;
    ext_init(e);
    if (P > 0 && !flat) {
        const int cn = Pm.cn;
        const size_t chanStride = (size_t)fc.dftH * hwp;
        const float2 *scr = a.ms.scratch[a.cls] + (size_t)slot * a.ms.scratchStride[a.cls];
        for (int k = 0; k < cn; k++) {
            const float2 *cb = scr + ((size_t)tileLocal * a.cnS + k) * chanStride;
            for (int p = 0; p < P; p++) {
                const int r = 2 * (pair0 + p);
                const float2 *sa = cb + (size_t)brev_bits(r, fc.log2H) * hwp;
                const float2 *sb = cb + (size_t)brev_bits(r + 1, fc.log2H) * hwp;
                float2 *zl = smem + p * ld;
                for (int kk = tid; kk < n; kk += nt) {
                    float2 z;
                    if (kk < hw) {
                        const float2 u = sa[kk], v = sb[kk];
                        z = make_float2(__fsub_rn(u.x, v.y), __fadd_rn(u.y, v.x));
                    } else {
                        const int mm = n - kk;
                        const float2 u = sa[mm], v = sb[mm];
                        z = make_float2(__fadd_rn(u.x, v.y), __fsub_rn(v.x, u.y));
                    }
                    zl[padi(brev_bits(kk, log2n))] = z;
                }
            }
            __syncthreads();
            auto la = [=](int line, int i) { return line * ld + padi(i); };
            fft_cascade<true>(smem, n, log2n, P, la, fc.triW);
            for (int p = 0; p < P; p++) {
                const float2 *zl = smem + p * ld;
                float *a0 = acc + (size_t)(2 * p) * n, *a1 = a0 + n;
                if (k == 0) {
                    for (int x = tid; x < bw; x += nt) {
                        const float2 z = zl[padi(x)];
                        a0[x] = z.x;
                        a1[x] = z.y;
                    }
                } else {
                    for (int x = tid; x < bw; x += nt) {
                        const float2 z = zl[padi(x)];
                        a0[x] = __fadd_rn(a0[x], z.x);
                        a1[x] = __fadd_rn(a1[x], z.y);
                    }
                }
            }
            __syncthreads();
        }
    }
    if (!a.ms.lanes) {
        // No statistics lanes: store the raw correlation for k_norm instead.
        if (P > 0 && !flat) {
            float *corr = a.ms.corr + (size_t)slot * a.ms.corrStride;
            for (int rr = 0; rr < 2 * P && 2 * pair0 + rr < bh; rr++)
                for (int x = tid; x < bw; x += nt)
                    corr[(size_t)(tb.y0 + 2 * pair0 + rr) * m.rw + tb.x0 + x] = acc[(size_t)rr * n + x];
        }
        return;
    }
    if (P > 0) {
        const float2 *lanes = a.ms.lanes + (size_t)slot * a.ms.lanesStride;
        float *map = a.ms.map;
        for (int rr = 0; rr < 2 * P; rr++) {
          const int r = 2 * pair0 + rr;
          if (r >= bh) break;
          for (int x = tid; x < bw; x += nt) {
            const long long li = (long long)(tb.y0 + r) * m.rw + tb.x0 + x;
            float score = 1.f;
            if (!flat) {
                const float2 td = lanes[li];
                const float num = __fsub_rn(acc[(size_t)rr * n + x], td.x);
                const float den = td.y, an = fabsf(num);
                if (an < den)
                    score = __fdiv_rn(num, den);
                else if (an < __fmul_rn(den, 1.125f))
                    score = num > 0.f ? 1.f : -1.f;
                else
                    score = 0.f;
            }
            if (map) map[li] = score;
            if (tb.y0 + r >= m.roiY0 && tb.y0 + r < m.roiY1 && tb.x0 + x >= m.roiX0 && tb.x0 + x < m.roiX1)
                ext_add(e, score, li);
          }
        }
    }
    __syncthreads();
    ext_block_reduce(e, shExt);
    if (tid == 0) {
        Partial &o = a.partials[m.partBase + a.partOffset + tileLocal * gridDim.x + blockIdx.x];
        o.minV = e.minV;
        o.maxV = e.maxV;
        o.minI = e.minI;
        o.maxI = e.maxI;
        __threadfence();
        isLast = atomicAdd(&a.counters[m.pIdx], 1) == a.nparts - 1;
    }
    __syncthreads();
    if (!isLast) return;
    __threadfence();
    ext_init(e);
    for (int i = tid; i < a.nparts; i += nt) {
        const volatile Partial *p = a.partials + m.partBase + i;
        Ext o;
        o.minV = p->minV;
        o.maxV = p->maxV;
        o.minI = p->minI;
        o.maxI = p->maxI;
        ext_merge(e, o);
    }
    __syncthreads();
    ext_block_reduce(e, shExt);
    if (tid == 0) ext_store_result(e, m.rw, a.out + m.outIdx);
}

// ----------------------------------------------------------- normalise

struct NormArgs {
    const uint8_t *img;
    long long istride;
    int step;
    MemberSet ms;
    int CW, BV, G, ncx, nby;
    int cnCap;            // channel capacity of the column arrays
    int cap;              // column capacity (>= CW + tw - 1 of every member)
    Partial *partials;
    int *counters;        // per member slot: CTAs finished (zeroed by the caller)
    cvm_result *out;
};


// Window statistics by the reference's own sliding scheme
// (colBuildGo/colSlideGo, impl.go:708-805, and the per-row window sums of
// impl.go:884-893), for a CW x BV block of results per CTA:
//   1. column sums over the th rows under the block (colBuildGo);
//   2. per group of G result rows, each thread slides its columns down
//      one row at a time (colSlideGo) and stores the per-row column sums;
//   3. one warp per row turns that row into an exclusive prefix over the
//      columns, so every window sum is one difference, and scores the row
//      with normOne (impl.go:825-849) against the raw correlation.
// All statistics are exact integers (u32 sums are modular: every window sum
// is < 2^32), so the schedule cannot change a value.  The CTA that
// finishes a member last merges the member's partial extrema in raster
// order (impl.go:1104-1112) and writes its result.
template <int CN>
__global__ void __launch_bounds__(256) k_norm(NormArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ Ext shExt[kThreads / 32];
    __shared__ int isLast;
    const int slot = blockIdx.z;
    const DevMember &m = member_of(a.ms, slot);
    const DevParams &Pm = a.ms.params[m.pIdx];
    if (Pm.cn != CN) return;  // this member belongs to the launch specialised on its cn
    const int X0 = blockIdx.x * a.CW, Y0 = blockIdx.y * a.BV;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
    Ext e;
    ext_init(e);
    const float *corr = a.ms.corr + (size_t)slot * a.ms.corrStride;
    float *map = a.ms.map;
    if (X0 < m.rw && Y0 < m.rh) {
        const int CWv = min(a.CW, m.rw - X0), Bv = min(a.BV, m.rh - Y0);
        if (Pm.flat) {
            for (int idx = tid; idx < CWv * Bv; idx += nt) {
                const int yy = idx / CWv, x = idx - yy * CWv;
                const long long li = (long long)(Y0 + yy) * m.rw + X0 + x;
                if (map) map[li] = 1.f;
                ext_add(e, 1.f, li);
            }
        } else {
            constexpr int cn = CN;
            const int tw = m.tw, th = m.th, step = a.step;
            const int NC = CWv + tw - 1;
            const int cap = a.cap, cnCap = a.cnCap, G = a.G;
            const int rcap = cap + 1;
            // shared layout: colQ[cap] u64 | rowQ[G][rcap] u64 | colS[cnCap][cap] u32 | rowS[cnCap][G][rcap] u32
            unsigned long long *colQ = reinterpret_cast<unsigned long long *>(smraw);
            unsigned long long *rowQ = colQ + cap;
            unsigned int *colS = reinterpret_cast<unsigned int *>(rowQ + (size_t)G * rcap);
            unsigned int *rowS = colS + (size_t)cnCap * cap;
            const long long area = (long long)tw * th;
            const unsigned int t0 = (unsigned int)Pm.tsum[0], t1 = (unsigned int)Pm.tsum[1];
            const unsigned int t2 = (unsigned int)Pm.tsum[2], t3 = (unsigned int)Pm.tsum[3];
            // 1. column sums over rows Y0 .. Y0+th-1
            for (int c = tid; c < NC; c += nt) {
                const uint8_t *p = a.img + (long long)Y0 * a.istride + (long long)(X0 + c) * step;
                unsigned int sk[4] = {0u, 0u, 0u, 0u};
                unsigned long long q = 0;
#pragma unroll 4
                for (int dy = 0; dy < th; dy++) {
                    const uint8_t *pr = p + (long long)dy * a.istride;
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        if (k < cn) {
                            const unsigned v = pr[k];
                            sk[k] += v;
                            q += v * v;
                        }
                }
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (k < cn) colS[(size_t)k * cap + c] = sk[k];
                colQ[c] = q;
            }
            __syncthreads();
            // lane chunks of the per-row scans; odd so lanes hit distinct banks
            const int chunk = ((NC + 1 + 31) / 32) | 1;
            for (int yg = Y0; yg < Y0 + Bv; yg += G) {
                const int Gv = min(G, Y0 + Bv - yg);
                // 2. per-row column sums of rows yg .. yg+Gv-1, sliding down
                for (int c = tid; c < NC; c += nt) {
                    unsigned int sk[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) sk[k] = k < cn ? colS[(size_t)k * cap + c] : 0u;
                    unsigned long long q = colQ[c];
                    const uint8_t *base = a.img + (long long)(X0 + c) * step;
                    for (int g = 0; g < Gv; g++) {
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            if (k < cn) rowS[((size_t)k * G + g) * rcap + c] = sk[k];
                        rowQ[(size_t)g * rcap + c] = q;
                        const int y = yg + g;
                        if (y + 1 < Y0 + Bv) {
                            const uint8_t *pa = base + (long long)(y + th) * a.istride;
                            const uint8_t *ps = base + (long long)y * a.istride;
                            long long dq = 0;
#pragma unroll
                            for (int k = 0; k < 4; k++)
                                if (k < cn) {
                                    const int va = pa[k], vb = ps[k];
                                    sk[k] += (unsigned int)(va - vb);
                                    dq += va * va - vb * vb;
                                }
                            q += (unsigned long long)dq;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        if (k < cn) colS[(size_t)k * cap + c] = sk[k];
                    colQ[c] = q;
                }
                __syncthreads();
                // 3. one warp per row: exclusive prefix, then the row's scores
                for (int g = warp; g < Gv; g += nw) {
                    unsigned int *rs[4];
#pragma unroll
                    for (int k = 0; k < 4; k++) rs[k] = rowS + ((size_t)k * G + g) * rcap;
                    unsigned long long *rq = rowQ + (size_t)g * rcap;
                    const int c0 = lane * chunk, c1 = min(NC, c0 + chunk);
                    unsigned int ls[4] = {0u, 0u, 0u, 0u};
                    unsigned long long lq = 0;
                    for (int c = c0; c < c1; c++) {
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            if (k < cn) ls[k] += rs[k][c];
                        lq += rq[c];
                    }
                    unsigned int xs[4];
                    unsigned long long xq = lq;
#pragma unroll
                    for (int k = 0; k < 4; k++) xs[k] = ls[k];
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const unsigned int u = __shfl_up_sync(0xffffffffu, xs[k], o);
                            if (lane >= o && k < cn) xs[k] += u;
                        }
                        const unsigned long long u = __shfl_up_sync(0xffffffffu, xq, o);
                        if (lane >= o) xq += u;
                    }
                    // exclusive offsets of this lane's chunk
#pragma unroll
                    for (int k = 0; k < 4; k++) xs[k] -= ls[k];
                    xq -= lq;
                    for (int c = c0; c < c1; c++) {
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            if (k < cn) {
                                const unsigned int v = rs[k][c];
                                rs[k][c] = xs[k];
                                xs[k] += v;
                            }
                        const unsigned long long v = rq[c];
                        rq[c] = xq;
                        xq += v;
                    }
                    if (c0 < NC && c1 == NC) {  // the lane ending the row stores prefix[NC]
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            if (k < cn) rs[k][NC] = xs[k];
                        rq[NC] = xq;
                    }
                    __syncwarp();
                    const int y = yg + g;
                    const float *crow = corr + (size_t)y * m.rw + X0;
                    for (int x = lane; x < CWv; x += 32) {
                        const unsigned int s0 = rs[0][x + tw] - rs[0][x];
                        unsigned long long cross = (unsigned long long)s0 * t0;
                        unsigned long long sq = (unsigned long long)s0 * s0;
                        if (cn > 1) {
                            const unsigned int s1 = rs[1][x + tw] - rs[1][x];
                            cross += (unsigned long long)s1 * t1;
                            sq += (unsigned long long)s1 * s1;
                        }
                        if (cn > 2) {
                            const unsigned int s2c = rs[2][x + tw] - rs[2][x];
                            cross += (unsigned long long)s2c * t2;
                            sq += (unsigned long long)s2c * s2c;
                        }
                        if (cn > 3) {
                            const unsigned int s3 = rs[3][x + tw] - rs[3][x];
                            cross += (unsigned long long)s3 * t3;
                            sq += (unsigned long long)s3 * s3;
                        }
                        const unsigned long long s2 = rq[x + tw] - rq[x];
                        const float l0 = cn == 1 ? __uint2float_rn(s0) : f32_via_f64((long long)cross);
                        const float id = f32_via_f64((long long)((unsigned long long)area * s2 - sq));
                        const float score = norm_one(crow[x], l0, id, s2, Pm.numScale, Pm.varScale, Pm.templNorm);
                        const long long li = (long long)y * m.rw + X0 + x;
                        if (map) map[li] = score;
                        ext_add(e, score, li);
                    }
                }
                __syncthreads();
            }
        }
    }
    __syncthreads();
    ext_block_reduce(e, shExt);
    const int nparts = a.ncx * a.nby;
    if (tid == 0) {
        Partial &o = a.partials[m.partBase + blockIdx.y * a.ncx + blockIdx.x];
        o.minV = e.minV;
        o.maxV = e.maxV;
        o.minI = e.minI;
        o.maxI = e.maxI;
        __threadfence();
        isLast = atomicAdd(&a.counters[m.pIdx], 1) == nparts - 1;
    }
    __syncthreads();
    if (!isLast) return;
    // The member's last CTA: merge all partials in raster-order semantics.
    __threadfence();
    ext_init(e);
    for (int i = tid; i < nparts; i += nt) {
        const volatile Partial *p = a.partials + m.partBase + i;
        Ext o;
        o.minV = p->minV;
        o.maxV = p->maxV;
        o.minI = p->minI;
        o.maxI = p->maxI;
        ext_merge(e, o);
    }
    __syncthreads();
    ext_block_reduce(e, shExt);
    if (tid == 0) ext_store_result(e, m.rw, a.out + m.outIdx);
}

// ------------------------------------------- separable window statistics

// Horizontal window sums of every image row for template width tw:
// H_q(x, r) = sum_{dx<tw} v_q(x+dx, r) for the CN channels and q = CN the
// squared pixels summed over the channels (impl.go:708-805 restated as a
// separable box sum).  One CTA per image row: a block prefix scan of the
// row in u32 (modular; every window sum is < 2^32 because tw <= 8192 and
// cn*65025*tw < 2^32), then one difference per output.  The cn+1 values
// of one (row, x) are interleaved, stat_pitch(cn) u32 apart per x, so a
// reader fetches them with one vector load: H[(r*hp + x)*pitch + q].
struct HsumArgs {
    const uint8_t *img;
    long long istride;
    int step, iw, ih, rw, tw, hp;
    unsigned int *H;          // wave slot z at H + z*slotStride
    size_t slotStride;
    const DevMember *table;   // fleet: per-slot member (tw, pIdx); nullptr: solo
    int first;
    const DevParams *params;
    int pIdx;                 // solo member params index
};

template <int CN>
__device__ __forceinline__ void hsum_row(const HsumArgs &a, int slot, int tw, int rw, unsigned int *sp,
                                         unsigned int (*wsum)[5]) {
    const int r = blockIdx.x, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int iw = a.iw, ld = iw + 1;
    const uint8_t *row = a.img + (long long)r * a.istride;
    // 1. coalesced staging of the row's channel values (slot c+1; slot 0 = 0)
    if (a.step == 4 && ((reinterpret_cast<size_t>(row) & 3) == 0)) {
        const uchar4 *r4 = reinterpret_cast<const uchar4 *>(row);
        for (int x = tid; x < iw; x += nt) {
            const uchar4 v = r4[x];
            const unsigned int c[4] = {v.x, v.y, v.z, v.w};
            unsigned int q = 0;
#pragma unroll
            for (int k = 0; k < CN; k++) {
                sp[k * ld + x + 1] = c[k];
                q += c[k] * c[k];
            }
            sp[CN * ld + x + 1] = q;
        }
    } else {
        for (int x = tid; x < iw; x += nt) {
            const uint8_t *p = row + (long long)x * a.step;
            unsigned int q = 0;
#pragma unroll
            for (int k = 0; k < CN; k++) {
                const unsigned int v = p[k];
                sp[k * ld + x + 1] = v;
                q += v * v;
            }
            sp[CN * ld + x + 1] = q;
        }
    }
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q <= CN; q++) sp[q * ld] = 0u;
    }
    __syncthreads();
    // 2. in-place inclusive prefix over slots 1..iw: odd-length segments keep
    //    the lanes on distinct banks
    const int seg = ((iw + nt - 1) / nt) | 1;
    const int c0 = 1 + tid * seg, c1 = min(iw + 1, c0 + seg);
    unsigned int tot[CN + 1];
#pragma unroll
    for (int q = 0; q <= CN; q++) tot[q] = 0u;
    for (int c = c0; c < c1; c++) {
#pragma unroll
        for (int q = 0; q <= CN; q++) tot[q] += sp[q * ld + c];
    }
    unsigned int inc[CN + 1];
#pragma unroll
    for (int q = 0; q <= CN; q++) inc[q] = tot[q];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q <= CN; q++) {
            const unsigned int u = __shfl_up_sync(0xffffffffu, inc[q], o);
            if (lane >= o) inc[q] += u;
        }
    }
    if (lane == 31) {
#pragma unroll
        for (int q = 0; q <= CN; q++) wsum[warp][q] = inc[q];
    }
    __syncthreads();
    unsigned int run[CN + 1];
#pragma unroll
    for (int q = 0; q <= CN; q++) {
        run[q] = inc[q] - tot[q];
        for (int w = 0; w < warp; w++) run[q] += wsum[w][q];
    }
    for (int c = c0; c < c1; c++) {
#pragma unroll
        for (int q = 0; q <= CN; q++) {
            run[q] += sp[q * ld + c];
            sp[q * ld + c] = run[q];
        }
    }
    __syncthreads();
    // 3. window sums, interleaved per x, one vector store each
    constexpr int NP = stat_pitch_c(CN);
    unsigned int *H = a.H + (size_t)slot * a.slotStride + (size_t)r * a.hp * NP;
    for (int x = tid; x < rw; x += nt) {
        unsigned int v[NP];
#pragma unroll
        for (int q = 0; q < NP; q++) v[q] = q <= CN ? sp[q * ld + x + tw] - sp[q * ld + x] : 0u;
        stv<NP>(H + (size_t)x * NP, v);
    }
}

// Exclusive row prefixes of one image row shared by every fleet member:
// planes 0..CN-1 the channel sums, plane CN the squares of the first
// min(CN,3) channels and, for CN == 4, plane 5 the alpha squares (a cn=3
// member's squared sum excludes alpha, a cn=4 member's includes it).
// Each member's window sum is then P[x+tw] - P[x] at its own width.
template <int CN>
__global__ void __launch_bounds__(256) k_row_prefix(const uint8_t *__restrict__ img, long long istride, int step,
                                                    int iw, unsigned int *P, int hp, size_t alphaOff) {
    constexpr int NQ = CN == 4 ? 6 : CN + 1;
    extern __shared__ __align__(16) unsigned int sp[];  // [NQ][iw+1]
    __shared__ unsigned int wsum[kThreads / 32][NQ];
    const int r = blockIdx.x, tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5;
    const int ld = iw + 1;
    const uint8_t *row = img + (long long)r * istride;
    for (int x = tid; x < iw; x += nt) {
        const uint8_t *p = row + (long long)x * step;
        unsigned int q3 = 0;
#pragma unroll
        for (int k = 0; k < CN; k++) {
            const unsigned int v = p[k];
            sp[k * ld + x + 1] = v;
            if (k < 3) q3 += v * v;
        }
        sp[CN * ld + x + 1] = q3;
        if (CN == 4) sp[5 * ld + x + 1] = (unsigned int)p[3] * p[3];
    }
    if (tid == 0) {
#pragma unroll
        for (int q = 0; q < NQ; q++) sp[q * ld] = 0u;
    }
    __syncthreads();
    const int seg = ((iw + nt - 1) / nt) | 1;
    const int c0 = 1 + tid * seg, c1 = min(iw + 1, c0 + seg);
    unsigned int tot[NQ], inc[NQ], run[NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) tot[q] = 0u;
    for (int c = c0; c < c1; c++) {
#pragma unroll
        for (int q = 0; q < NQ; q++) tot[q] += sp[q * ld + c];
    }
#pragma unroll
    for (int q = 0; q < NQ; q++) inc[q] = tot[q];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            const unsigned int u = __shfl_up_sync(0xffffffffu, inc[q], o);
            if (lane >= o) inc[q] += u;
        }
    }
    if (lane == 31) {
#pragma unroll
        for (int q = 0; q < NQ; q++) wsum[warp][q] = inc[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        run[q] = inc[q] - tot[q];
        for (int w = 0; w < warp; w++) run[q] += wsum[w][q];
    }
    for (int c = c0; c < c1; c++) {
#pragma unroll
        for (int q = 0; q < NQ; q++) {
            run[q] += sp[q * ld + c];
            sp[q * ld + c] = run[q];
        }
    }
    __syncthreads();
    // CN < 4: the CN+1 values interleaved per x (pitch stat_pitch(CN));
    // CN == 4: (s0, s1, s2, RGB squares) per x, and (s3, alpha squares) per x
    // in a second block at alphaOff, so 3-channel readers load 16 bytes
    constexpr int NP = CN == 4 ? 4 : stat_pitch_c(CN);
    unsigned int *out = P + (size_t)r * hp * NP;
    for (int x = tid; x <= iw; x += nt) {
        unsigned int v[NP];
        if (CN == 4) {
            v[0] = sp[x];
            v[1] = sp[ld + x];
            v[2] = sp[2 * ld + x];
            v[3] = sp[4 * ld + x];
        } else {
#pragma unroll
            for (int q = 0; q < NP; q++) v[q] = q < NQ ? sp[q * ld + x] : 0u;
        }
        stv<NP>(out + (size_t)x * NP, v);
        if (CN == 4) {
            const unsigned int w[2] = {sp[3 * ld + x], sp[5 * ld + x]};
            stv<2>(P + alphaOff + ((size_t)r * hp + x) * 2, w);
        }
    }
}

// One launch covers members of either channel count of a mode (colour: 3
// or 4, chosen on the device; gray: 1).
template <int CNA, int CNB>
__global__ void __launch_bounds__(256) k_hsum(HsumArgs a) {
    extern __shared__ __align__(16) unsigned int sp[];  // [cn+1][iw+1]
    __shared__ unsigned int wsum[kThreads / 32][5];
    const int slot = blockIdx.z;
    int tw = a.tw, rw = a.rw, pIdx = a.pIdx;
    if (a.table) {
        const DevMember &m = a.table[a.first + slot];
        tw = m.tw;
        rw = m.rw;
        pIdx = m.pIdx;
    }
    const DevParams &Pm = a.params[pIdx];
    if (Pm.flat) return;
    if (Pm.cn == CNA)
        hsum_row<CNA>(a, slot, tw, rw, sp, wsum);
    else if (CNB != CNA && Pm.cn == CNB)
        hsum_row<CNB>(a, slot, tw, rw, sp, wsum);
}

// Vertical sliding of the horizontal window sums, one thread per result
// column over a band of BV rows: the window statistics of (x, y) are
// sum_{dy<th} H(x, y+dy), updated by one entering and one leaving row per
// step.  Everything of normOne (impl.go:825-849) that does not involve the
// correlation is evaluated here and stored per result as
//   t   = float32(lane0) * numScale
//   den = sqrt(idiff * varScale) * templNorm, or 0 under the lim guard
// so the inverse-rows epilogue only needs num = corr - t and the ladder.
struct VstatArgs {
    const unsigned int *H;    // per-slot window sums, or (PRE) the shared row prefix
    size_t slotStride;
    size_t alphaOff;          // PRE with a 4-channel prefix: the (s3, alpha squares) block
    int hp;
    MemberSet ms;
    int BV;
    // one match with a tall template: the window sums summed over 16-row
    // blocks (row b = H rows 16b .. 16b+15, H's layout), so a band starts
    // from th/16 block rows and at most 15 single rows (nullptr: none)
    const unsigned int *blk;
};

// The 16-row block sums of one match's horizontal window sums (u32,
// modular like H: every sum the slide forms from them is exact).
__global__ void k_vblock(const unsigned int *__restrict__ H, unsigned int *__restrict__ B, int nblk,
                         size_t rowElems) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = blockIdx.y;
    if (e >= rowElems || b >= nblk) return;
    const unsigned int *h = H + (size_t)b * 16 * rowElems + e;
    unsigned int v[16];
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __ldg(h + (size_t)i * rowElems);
    unsigned int sum = 0u;
#pragma unroll
    for (int i = 0; i < 16; i++) sum += v[i];
    B[(size_t)b * rowElems + e] = sum;
}

// The frame's summed-area table over the shared row prefix's lanes,
// S[y][e] = sum_{r < y} P[r][e] for y = 0 .. rows (u32, modulo 2^32 like
// the prefix), in three steps: 16-row block sums, their exclusive scan down
// each lane (the total in block nb), then each block's rows from its start.
__global__ void k_sat_blocks(const unsigned int *__restrict__ P, int rows, size_t rowElems,
                             unsigned int *__restrict__ B) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rowElems) return;
    const int r0 = 16 * blockIdx.y, n = min(16, rows - r0);
    const unsigned int *p = P + (size_t)r0 * rowElems + e;
    unsigned int v[16];
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = i < n ? __ldg(p + (size_t)i * rowElems) : 0u;
    unsigned int sum = 0u;
#pragma unroll
    for (int i = 0; i < 16; i++) sum += v[i];
    B[(size_t)blockIdx.y * rowElems + e] = sum;
}

__global__ void k_sat_scan(unsigned int *B, int nb, size_t rowElems) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rowElems) return;
    unsigned int run = 0u;
    for (int b0 = 0; b0 < nb; b0 += 8) {
        unsigned int v[8];
#pragma unroll
        for (int i = 0; i < 8; i++) v[i] = b0 + i < nb ? B[(size_t)(b0 + i) * rowElems + e] : 0u;
#pragma unroll
        for (int i = 0; i < 8; i++)
            if (b0 + i < nb) {
                B[(size_t)(b0 + i) * rowElems + e] = run;
                run += v[i];
            }
    }
    B[(size_t)nb * rowElems + e] = run;
}

__global__ void k_sat_fill(const unsigned int *__restrict__ P, int rows, size_t rowElems,
                           const unsigned int *__restrict__ B, unsigned int *__restrict__ S) {
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= rowElems) return;
    const int r0 = 16 * blockIdx.y;
    if (r0 > rows) return;
    const int n = min(16, rows - r0);  // prefix rows added inside this block
    const unsigned int *p = P + (size_t)r0 * rowElems + e;
    unsigned int v[16];
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = i < n ? __ldg(p + (size_t)i * rowElems) : 0u;
    unsigned int run = B[(size_t)blockIdx.y * rowElems + e];
    unsigned int *s = S + (size_t)r0 * rowElems + e;
#pragma unroll
    for (int i = 0; i < 16; i++) {
        if (r0 + i > rows) break;
        s[(size_t)i * rowElems] = run;
        run += v[i];
    }
}

// PRE: H is the shared row prefix built for PCN channels (window sum =
// P[x+tw] - P[x]); its squares are plane PCN (PCN < 4) or planes 4 (RGB)
// and 5 (alpha) when PCN == 4 (a cn = 3 member leaves alpha out).
// FAST (the fleet's fast form, zero-mean template spectra): the
// correlation already is the numerator, so only den is stored, one float
// per result (the first half of the member's lanes slot).
template <int CN, bool PRE, int PCN, bool FAST = false>
__device__ __forceinline__ void vstat_cols(const VstatArgs &a, const DevMember &m, const DevParams &Pm) {
    constexpr int NP = PRE ? (PCN == 4 ? 4 : stat_pitch_c(PCN)) : stat_pitch_c(CN);
    // PRE (a fleet wave): members vary fastest across the grid, so the
    // CTAs resident together read the same prefix region and share it in L2
    const int slot = PRE ? blockIdx.x : blockIdx.z;
    const int x = (PRE ? blockIdx.y : blockIdx.x) * blockDim.x + threadIdx.x;
    const int Y0 = (PRE ? blockIdx.z : blockIdx.y) * a.BV;
    if (x >= m.rw || Y0 >= m.rh) return;
    // results outside the member's region of interest are never read
    if (a.ms.anyRoi && (x < m.roiX0 || x >= m.roiX1 || Y0 >= m.roiY1 || Y0 + a.BV <= m.roiY0)) return;
    const int Bv = min(a.BV, m.rh - Y0);
    const int th = m.th;
    const size_t rp = (size_t)a.hp * NP;  // row pitch
    const unsigned int *H = a.H + (PRE ? 0 : (size_t)slot * a.slotStride) + (size_t)x * NP;
    const int twoff = PRE ? m.tw * NP : 0;
    float2 *lanes = a.ms.lanes + (size_t)slot * a.ms.lanesStride + x;
    float *dens = reinterpret_cast<float *>(a.ms.lanes + (size_t)slot * a.ms.lanesStride) + x;
    // the CN sums and the squared sum of row h's window
    auto rowvals = [&](const unsigned int *h, unsigned int *hv) {
        unsigned int A[NP];
        ldv<NP>(A, h + twoff);
        if (!PRE) {
#pragma unroll
            for (int q = 0; q <= CN; q++) hv[q] = A[q];
        } else {
            unsigned int Bq[NP];
            ldv<NP>(Bq, h);
#pragma unroll
            if (PCN == 4) {
#pragma unroll
                for (int q = 0; q < 3; q++) hv[q] = A[q] - Bq[q];
                if (CN == 4) {
                    // the alpha block: same row and column, pitch 2
                    const unsigned int *ha = a.H + a.alphaOff + (size_t)(h - H) / NP * 2 + (size_t)x * 2;
                    unsigned int A2[2], B2[2];
                    ldv<2>(A2, ha + 2 * m.tw);
                    ldv<2>(B2, ha);
                    hv[3] = A2[0] - B2[0];
                    hv[CN] = (A[3] - Bq[3]) + (A2[1] - B2[1]);
                } else {
                    hv[CN] = A[3] - Bq[3];
                }
            } else {
#pragma unroll
                for (int q = 0; q < CN; q++) hv[q] = A[q] - Bq[q];
                hv[CN] = A[PCN] - Bq[PCN];
            }
        }
    };
    unsigned int s[CN];
    unsigned long long q = 0;
#pragma unroll
    for (int k = 0; k < CN; k++) s[k] = 0u;
    int dy0 = 0;
    // (a fleet's block sums cover the main prefix block only: members whose
    // squared sum needs the alpha block start row by row)
    if (a.blk && !(PRE && PCN == 4 && CN == 4)) {
        // whole 16-row blocks first (Y0 is a multiple of 16: BV is)
        const unsigned int *Bx = a.blk + (size_t)x * NP;
#pragma unroll 4
        for (; dy0 + 16 <= th; dy0 += 16) {
            unsigned int hv[CN + 1];
            rowvals(Bx + (size_t)((Y0 + dy0) >> 4) * rp, hv);
#pragma unroll
            for (int k = 0; k < CN; k++) s[k] += hv[k];
            q += hv[CN];
        }
    }
#pragma unroll(PRE ? 4 : 8)
    for (int dy = dy0; dy < th; dy++) {
        unsigned int hv[CN + 1];
        rowvals(H + (size_t)(Y0 + dy) * rp, hv);
#pragma unroll
        for (int k = 0; k < CN; k++) s[k] += hv[k];
        q += hv[CN];
    }
    const unsigned long long area = (unsigned long long)m.tw * th;
    const unsigned int t0 = (unsigned int)Pm.tsum[0], t1 = (unsigned int)Pm.tsum[1];
    const unsigned int t2 = (unsigned int)Pm.tsum[2], t3 = (unsigned int)Pm.tsum[3];
    const float eps = 1.1920928955078125e-06f;  // 10 * 2^-23
    // The slide in batches of RB rows: every row the batch enters and leaves
    // is loaded first (2 * RB row loads in flight), then the batch's results
    // are scored in order -- one wait on L2 per batch instead of per row.
    // A fleet's prefix differences (two loads per row) keep RB = 1: the
    // batch's registers cost more occupancy than its loads in flight gain.
    constexpr int RB = PRE ? 1 : 4;
    for (int yb = Y0; yb < Y0 + Bv; yb += RB) {
        unsigned int hinB[RB][CN + 1], houtB[RB][CN + 1];
#pragma unroll
        for (int r = 0; r < RB; r++)
            if (yb + r + 1 < Y0 + Bv) {
                rowvals(H + (size_t)(yb + r + th) * rp, hinB[r]);
                rowvals(H + (size_t)(yb + r) * rp, houtB[r]);
            }
#pragma unroll
        for (int r = 0; r < RB; r++) {
            const int y = yb + r;
            if (y >= Y0 + Bv) break;
            const bool more = y + 1 < Y0 + Bv;
            const unsigned int *hin = hinB[r], *hout = houtB[r];
            unsigned long long cross = 0, sq = (unsigned long long)s[0] * s[0];
            if (!FAST) cross = (unsigned long long)s[0] * t0;
            if (CN > 1) {
                if (!FAST) cross += (unsigned long long)s[CN > 1 ? 1 : 0] * t1;
                sq += (unsigned long long)s[CN > 1 ? 1 : 0] * s[CN > 1 ? 1 : 0];
            }
            if (CN > 2) {
                if (!FAST) cross += (unsigned long long)s[CN > 2 ? 2 : 0] * t2;
                sq += (unsigned long long)s[CN > 2 ? 2 : 0] * s[CN > 2 ? 2 : 0];
            }
            if (CN > 3) {
                if (!FAST) cross += (unsigned long long)s[CN > 3 ? 3 : 0] * t3;
                sq += (unsigned long long)s[CN > 3 ? 3 : 0] * s[CN > 3 ? 3 : 0];
            }
            // the spill lanes (impl.go:902-1009) and normOne's corr-free part
            // FAST: the exact variance numerator from its two 32-bit halves
            // (within 1.5 ulp; the reference's two-step float64 -> float32
            // conversion is kept otherwise)
            const unsigned long long idv = area * q - sq;
            const float id = FAST ? fmaf(__uint2float_rn((unsigned int)(idv >> 32)), 4294967296.0f,
                                         __uint2float_rn((unsigned int)idv))
                                  : f32_via_f64((long long)idv);
            const float diff2 = __fmul_rn(id, Pm.varScale);
            float lim = 0.5f;
            if (q < (1ull << 24)) {
                lim = __fmul_rn(eps, __uint2float_rn((unsigned int)q));
                if (lim > 0.5f) lim = 0.5f;
            }
            // FAST: the square root from the hardware reciprocal square root
            // (within 2 ulp) instead of the correctly rounded sequence
            const float sd = FAST ? __fmul_rn(diff2, rsqrtf(diff2)) : __fsqrt_rn(diff2);
            const float den = diff2 > lim ? __fmul_rn(sd, Pm.templNorm) : 0.f;
            if (FAST) {
                dens[(size_t)y * m.rw] = den;
            } else {
                const float l0 = CN == 1 ? __uint2float_rn(s[0]) : f32_via_f64((long long)cross);
                lanes[(size_t)y * m.rw] = make_float2(__fmul_rn(l0, Pm.numScale), den);
            }
            if (more) {
#pragma unroll
                for (int k = 0; k < CN; k++) s[k] += hin[k] - hout[k];
                q += (unsigned long long)hin[CN] - (unsigned long long)hout[CN];
            }
        }
    }
}

template <int CNA, int CNB, bool PRE, bool FAST = false>
__global__ void __launch_bounds__(256) k_vstats(VstatArgs a) {
    const DevMember &m = member_of(a.ms, PRE ? blockIdx.x : blockIdx.z);
    const DevParams &Pm = a.ms.params[m.pIdx];
    if (Pm.flat) return;
    if (Pm.cn == CNA)
        vstat_cols<CNA, PRE, CNB, FAST>(a, m, Pm);
    else if (CNB != CNA && Pm.cn == CNB)
        vstat_cols<CNB, PRE, CNB, FAST>(a, m, Pm);
}

// Frame ingest from page-locked host memory: the GPU reads the caller's
// rows over the host link directly (many 16-byte loads in flight per
// thread), instead of the copy engine's single stream of transfers.
template <typename V>
__global__ void k_ingest(unsigned char *__restrict__ dst, size_t dpitch, const unsigned char *__restrict__ src,
                         size_t spitch, int perRow, int rows) {
    const long long items = (long long)perRow * rows;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; i0 < items; i0 += 4 * stride) {
        V v[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const long long i = i0 + k * stride;
            if (i < items) {
                const long long y = i / perRow, x = i - y * perRow;
                v[k] = reinterpret_cast<const V *>(src + y * spitch)[x];
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const long long i = i0 + k * stride;
            if (i < items) {
                const long long y = i / perRow, x = i - y * perRow;
                reinterpret_cast<V *>(dst + y * dpitch)[x] = v[k];
            }
        }
    }
}

// Small host values to device memory through kernel arguments.
struct UploadBlob {
    unsigned char bytes[3072];
};

__global__ void k_upload(unsigned char *dst, UploadBlob b, int n) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = b.bytes[i];
}

// shrinkInto (impl.go:591-610): the shrunk band's spectrum is the
// stride-2^s row gather of the full one times 2^s (exact).
__global__ void k_shrink_gather(const float2 *__restrict__ src, int dftH, float2 *__restrict__ dst,
                                int dh2, int hwp, int cnS) {
    const int shift = __ffs(dftH) - __ffs(dh2);
    const float up = (float)(1 << shift);
    const long long total = (long long)cnS * dh2 * hwp;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % hwp);
        const long long kr = i / hwp;
        const int r = (int)(kr % dh2), k = (int)(kr / dh2);
        const float2 v = src[((size_t)k * dftH + ((size_t)r << shift)) * hwp + x];
        dst[i] = make_float2(__fmul_rn(v.x, up), __fmul_rn(v.y, up));
    }
}


int ilog2i(int v) {
    int l = 0;
    while ((1 << l) < v) l++;
    return l;
}

}  // namespace

// ------------------------------------------------------------- launches

cudaError_t launch_gray(const uint8_t *src, long long sstride, int w, int h, uint8_t *dst,
                        long long dstride, cudaStream_t st) {
    dim3 grid((w + kThreads - 1) / kThreads, h);
    ProfScope ps("k_gray", st);
    k_gray<<<grid, kThreads, 0, st>>>(src, sstride, w, h, dst, dstride);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_alpha_scan(const uint8_t *img, long long stride, int w, int h,
                              unsigned int *mismatch, cudaStream_t st) {
    dim3 grid((w + kThreads - 1) / kThreads, h);
    ProfScope ps("k_alpha_scan", st);
    k_alpha_scan<<<grid, kThreads, 0, st>>>(img, stride, w, h, mismatch);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_prep(const uint8_t *tpl, long long tstride, int tw, int th, int tstep, int cnStats,
                        const uint8_t *parent, long long pstride, int pw, int ph, DevParams *P, int n,
                        int setInit, int initMode, int initCnFixed, DevFrame *F, cudaStream_t st) {
    PrepArgs a;
    a.tpl = tpl;
    a.tstride = tstride;
    a.tw = tw;
    a.th = th;
    a.tstep = tstep;
    a.cnStats = cnStats;
    a.tplCtas = 0;
    if (tpl) {
        const long long total = (long long)tw * th;
        long long c = (total + 4 * kThreads - 1) / (4 * kThreads);
        a.tplCtas = (int)(c < 1 ? 1 : (c > 128 ? 128 : c));
    }
    a.parent = parent;
    a.pstride = pstride;
    a.pw = pw;
    a.ph = ph;
    a.parentCtas = parent ? (ph < 304 ? ph : 304) : 0;
    a.pvec16 = parent && (reinterpret_cast<uintptr_t>(parent) & 15) == 0 && (pstride & 15) == 0;
    a.P = P;
    a.n = n;
    a.setInit = setInit;
    a.initMode = initMode;
    a.initCnFixed = initCnFixed;
    a.F = F;
    int grid = a.tplCtas + a.parentCtas;
    if (grid < 1) grid = 1;
    ProfScope ps("k_prep", st);
    k_prep<<<grid, kThreads, 0, st>>>(a);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_fwd_rows(const uint8_t *img, long long istride, int step, int chanCount,
                            const int *cnDev, const TileGeom &g, const FftClass &fc, float2 *spec,
                            int cnS, cudaStream_t st, int chanFirst, const char *label, float mul,
                            const float *sub, const unsigned long long *subSums, float subDiv, int selfSums) {
    // Channels per launch so that one row pair of the group fits 128 KB of
    // shared memory; row pairs per CTA fill ~32 KB when rows are short.
    int group = 16384 / fc.n;
    if (group < 1) group = 1;
    if (group > chanCount - chanFirst) group = chanCount - chanFirst;
    int P = 4096 / (fc.n * group);
    if (P < 1) P = 1;
    // Largest row count of any tile: blockH + thL - 1, capped by dftH.
    int maxRows = g.blockH + g.thL - 1;
    if (maxRows > fc.dftH) maxRows = fc.dftH;
    const int pairs = (maxRows + 1) / 2;
    // few rows (a small template or frame): fewer pairs per CTA until the
    // launch has a CTA per SM, so the rows are spread over the SMs
    while (P > 1 && (long long)((pairs + P - 1) / P) * fc.ntiles < 152) P >>= 1;
    dim3 grid((pairs + P - 1) / P, fc.ntiles);
    const size_t smem = (size_t)P * group * padded_len(fc.n) * sizeof(float2);
    // as many threads as a radix-16 pass has units (a multiple of 32 in
    // 64..256), so no thread idles in those passes; a device-chosen colour
    // count is 3 unless an alpha plane varies, so size for that
    const int groupLikely = (cnDev && chanCount == 4 && group == 4) ? 3 : group;
    int threads = P * groupLikely * (fc.n >= 16 ? fc.n / 16 : 1);
    threads = threads < 64 ? 64 : (threads > kThreads ? kThreads : (threads + 31) / 32 * 32);
    if (rows_fixed_length(fc.log2n)) {
        FwdRowsArgs a;
        a.img = img;
        a.istride = istride;
        a.step = step;
        a.chanCount = chanCount;
        a.cnDev = cnDev;
        a.chanGroup = group;
        a.g = g;
        a.fc = fc;
        a.spec = spec;
        a.cnS = cnS;
        a.pairsPerCta = P;
        a.pix32 = step == 4 && (reinterpret_cast<uintptr_t>(img) & 3) == 0 && (istride & 3) == 0;
        a.mul = mul;
        for (int k = 0; k < 4; k++) a.sub[k] = sub ? sub[k] : 0.0f;
        a.subSums = subSums;
        a.subDiv = subDiv;
        a.selfSums = selfSums;
        // a sample transform marks the fast form (the exact form packs the
        // reference's samples untouched): its butterflies may fuse
        a.fma = (mul != 1.0f || sub || subSums || selfSums) ? 1 : 0;
        // Frames of 4-byte or gray pixels at 16-byte aligned addresses and
        // pitches are staged by TMA: each CTA's rows in boxes of 256 bytes
        // after the line buffers (the widest tile's span + the 16-byte
        // rounding, per box row).  Frame extent: the tiles' loads lie inside
        // the rows/columns the geometry covers (x0 + loadW <= rwT + twL - 1).
        CUtensorMap map;
        memset(&map, 0, sizeof map);
        a.tma = 0;
        a.tmaSmemOff = 0;
        size_t smemT = smem;
        const int maxLoadW = std::min(fc.n, g.blockW + g.twL - 1);
        const long long wBytes = (long long)(g.rwT + g.twL - 1) * step;
        const int hRows = g.rhT + g.thL - 1;
        if (!selfSums && (step == 4 ? a.pix32 : step == 1) && (reinterpret_cast<uintptr_t>(img) & 15) == 0 &&
            (istride & 15) == 0 && 2 * P <= 256 && fc.n >= 256) {
            const int nbMax = (15 + maxLoadW * step + 255) / 256;
            const size_t off = (smem + 127) / 128 * 128;
            const size_t need = off + 128 + (size_t)nbMax * 256 * 2 * P;  // + the kernel's runtime alignment
            if (need <= 200 * 1024 && encode_frame_map(&map, img, istride, wBytes, hRows, 2 * P)) {
                a.tma = 1;
                a.tmaSmemOff = (unsigned)off;
                smemT = need;
            }
        }
        ProfScope ps(label ? label : (a.tma ? "k_fwd_rows_tma" : "k_fwd_rows"), st);
        for (int c0 = chanFirst; c0 < chanCount; c0 += group) {
            a.chanFirst = c0;
            launch_fwd_rows_fixed(a, map, grid, threads, smemT, st);
            count_launches(1);
        }
        return cudaGetLastError();
    }
    ProfScope ps(label ? label : "k_fwd_rows", st);
    if (mul != 1.0f || sub || subSums || selfSums) return cudaErrorInvalidValue;  // sample transform: fixed lengths only
    set_smem(k_fwd_rows, smem);
    for (int c0 = chanFirst; c0 < chanCount; c0 += group) {
        k_fwd_rows<<<grid, threads, smem, st>>>(img, istride, step, chanCount, cnDev, c0, group, g, fc,
                                                 spec, cnS, P);
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_cols(int mode, const float2 *in, float2 *out, int cnS, const TileGeom &g,
                        const FftClass &fc, int cls, int chanCount, const int *cnDev, float scale,
                        const MemberSet &ms, int nmembers, cudaStream_t st, const char *label) {
    ColsArgs a;
    a.mode = mode;
    a.in = in;
    a.out = out;
    a.cnS = cnS;
    a.g = g;
    a.fc = fc;
    a.cls = cls;
    a.chanCount = chanCount;
    a.cnDev = cnDev;
    a.scale = scale;
    a.ms = ms;
    a.nmem = mode == 0 ? 1 : nmembers;
    int SC = 8192 / fc.dftH;
    if (SC > 16) SC = 16;
    if (SC < 1) SC = 1;
    a.SC = SC;
    a.logSC = ilog2i(SC);
    // the generic kernels take (strip, channel, tile x member); the fixed
    // heights' fleet modes take (tile x member, channel, strip)
    const int strips = (fc.hw + SC - 1) / SC;
    dim3 grid(strips, chanCount, fc.ntiles * (mode == 0 ? 1 : nmembers));
    if (mode >= 2 && cols_fixed_length(fc.log2H)) grid = dim3(fc.ntiles * nmembers, mode == 3 ? 1 : chanCount, strips);
    const size_t smem = (size_t)fc.dftH * SC * sizeof(float2);
    ProfScope ps(label ? label
                       : (mode == 0 ? "k_cols_fwd"
                                    : (mode == 1 ? "k_cols_fwd_mul_inv"
                                                 : (mode == 2 ? "k_cols_mul_inv"
                                                              : (mode == 3 ? "k_cols_sum_inv" : "k_cols_fwd_sum_inv")))),
                 st);
    if (mode == 3 && !cols_fixed_length(fc.log2H)) return cudaErrorInvalidValue;  // fast form: fixed heights only
    if (mode == 4) {
        // every channel of a strip in one CTA (cnS strips of dftH x SC)
        if (!cols_fixed_length(fc.log2H) || nmembers != 1 || ms.table) return cudaErrorInvalidValue;
        a.SC = cols_sum_width(fc.log2H);
        a.logSC = ilog2i(a.SC);
        const dim3 g4((fc.hw + a.SC - 1) / a.SC, 1, fc.ntiles);
        launch_cols_sum(a, g4, (size_t)cnS * fc.dftH * a.SC * sizeof(float2), st);
        count_launches(1);
        return cudaGetLastError();
    }
    if (cols_fixed_length(fc.log2H)) {
        launch_cols_fixed(a, grid, smem, st);
    } else if ((fc.log2H & 1) == 0 && fc.dftH >= 4) {
        if (mode == 0) {
            set_smem(k_cols_even<0>, smem);
            k_cols_even<0><<<grid, kThreads, smem, st>>>(a);
        } else if (mode == 1) {
            set_smem(k_cols_even<1>, smem);
            k_cols_even<1><<<grid, kThreads, smem, st>>>(a);
        } else {
            set_smem(k_cols_even<2>, smem);
            k_cols_even<2><<<grid, kThreads, smem, st>>>(a);
        }
    } else {
        set_smem(k_cols, smem);
        k_cols<<<grid, kThreads, smem, st>>>(a);
    }
    count_launches(1);
    return cudaGetLastError();
}

int inv_rows_ctas_per_tile(const FftClass &fc, int rowsMax, int *pairsPerCta, int wide, int tc) {
    // 4096 elements per CTA: the radix-16 passes (n/16 units per line) keep
    // all 256 threads busy, ~68 KB of shared memory (three CTAs per SM);
    // wide: 8192 elements (two units per thread per pass), ~70 KB without
    // the accumulator; the tensor-core kernel takes the same
    // (the tensor-core kernel keeps 8192: 32 pairs per CTA measured slower
    // for it, 6.25 against 5.14 ms per 256-member frame, and 4 pairs too)
    int P = (wide ? (tc ? 8192 : rows_fast_wave_elems(fc.log2n)) : 4096) / fc.n;
    if (P < 1) P = 1;
    // A tile emits at most rowsMax rows, and never more than dftH (a fleet
    // member's last band extends to its own result edge, still inside the
    // loaded rows <= dftH).  No CTA without rows: an idle CTA still takes an
    // SM slot, and a third CTA on an SM makes that SM the kernel's tail.
    const int rows = rowsMax < fc.dftH ? rowsMax : fc.dftH;
    const int pairs = (rows + 1) / 2;
    *pairsPerCta = P;
    return (pairs + P - 1) / P;
}

cudaError_t launch_inv_rows(const TileGeom &g, const FftClass &fc, int cls, int cnS, const MemberSet &ms,
                            int nmembers, int rowsMax, int partOffset, int nparts, Partial *partials, int *counters,
                            cvm_result *out, cudaStream_t st, int wide) {
    InvArgs a;
    a.g = g;
    a.fc = fc;
    a.cls = cls;
    a.cnS = cnS;
    a.ms = ms;
    int P = 0;
    if (wide && (!ms.form || !rows_fixed_length(fc.log2n))) return cudaErrorInvalidValue;
    const bool tc = inv_rows_tc_applies(fc, ms);
    const int ctas = inv_rows_ctas_per_tile(fc, rowsMax, &P, wide, tc);
    a.pairsPerCta = P;
    a.partOffset = partOffset;
    a.nparts = nparts;
    a.partials = partials;
    a.counters = counters;
    a.out = out;
    dim3 grid(ctas, fc.ntiles, nmembers);
    if (tc) {
        ProfScope ps("k_inv_rows_tc", st);
        const cudaError_t e = launch_inv_rows_tc(a, grid, st);
        count_launches(1);
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    const size_t smem = (size_t)P * (padded_len(fc.n) * sizeof(float2) + (wide ? 0 : 2 * fc.n * sizeof(float)));
    ProfScope ps("k_inv_rows", st);
    if (rows_fixed_length(fc.log2n)) {
        launch_inv_rows_fixed(a, grid, smem, st);
    } else {
        set_smem(k_inv_rows, smem);
        k_inv_rows<<<grid, kThreads, smem, st>>>(a);
    }
    count_launches(1);
    return cudaGetLastError();
}

static size_t norm_smem_bytes(int cap, int cnCap, int G) {
    return (size_t)cap * (8 + 4 * cnCap) + (size_t)G * (cap + 1) * (8 + 4 * cnCap);
}

NormGrid norm_grid(int rwMax, int rhMax, int twMax, int cnCap) {
    NormGrid g;
    g.CW = kThreads;
    g.B = 32;
    g.cnCap = cnCap;
    g.ncCap = g.CW + twMax - 1;
    g.G = 8;
    while (g.G > 1 && norm_smem_bytes(g.ncCap, cnCap, g.G) > 96 * 1024) g.G >>= 1;
    if (norm_smem_bytes(g.ncCap, cnCap, g.G) > 200 * 1024) {
        g.CW = 128;
        g.ncCap = g.CW + twMax - 1;
    }
    g.ncx = (rwMax + g.CW - 1) / g.CW;
    g.nby = (rhMax + g.B - 1) / g.B;
    g.smemBytes = norm_smem_bytes(g.ncCap, cnCap, g.G);
    g.scratchPerCta = 0;
    return g;
}

cudaError_t launch_norm(const uint8_t *img, long long istride, int step, const MemberSet &ms, int nmembers,
                        const NormGrid &ng, int cnLaunch, Partial *partials, int *counters, cvm_result *out,
                        cudaStream_t st) {
    NormArgs a;
    a.img = img;
    a.istride = istride;
    a.step = step;
    a.ms = ms;
    a.CW = ng.CW;
    a.BV = ng.B;
    a.G = ng.G;
    a.ncx = ng.ncx;
    a.nby = ng.nby;
    a.cnCap = ng.cnCap;
    a.cap = ng.ncCap;
    a.partials = partials;
    a.counters = counters;
    a.out = out;
    dim3 grid(ng.ncx, ng.nby, nmembers);
    ProfScope ps("k_norm", st);
    switch (cnLaunch) {
        case 1:
            set_smem(k_norm<1>, ng.smemBytes);
            k_norm<1><<<grid, kThreads, ng.smemBytes, st>>>(a);
            break;
        case 2:
            set_smem(k_norm<2>, ng.smemBytes);
            k_norm<2><<<grid, kThreads, ng.smemBytes, st>>>(a);
            break;
        case 3:
            set_smem(k_norm<3>, ng.smemBytes);
            k_norm<3><<<grid, kThreads, ng.smemBytes, st>>>(a);
            break;
        default:
            set_smem(k_norm<4>, ng.smemBytes);
            k_norm<4><<<grid, kThreads, ng.smemBytes, st>>>(a);
            break;
    }
    count_launches(1);
    return cudaGetLastError();
}

SepGrid sep_grid(int rwMax, int rhMax) {
    SepGrid g;
    g.BV = 16;
    g.ncx = (rwMax + kThreads - 1) / kThreads;
    g.nby = (rhMax + g.BV - 1) / g.BV;
    g.hp = (rwMax + 31) / 32 * 32;
    g.rhMax = rhMax;
    return g;
}

// Band height of the vertical slide: every band first sums th rows, so
// taller bands amortise that start over more results; the band stays at 16
// rows unless the launch has CTAs to spare (~6 per SM at the taller band),
// and at most 256 (a 78-member wave of 2560x1440 statistics: bands of 128
// rows 3.03 ms, 256 rows 2.91, 512 rows 3.09, 1024 rows 3.61 -- the
// tallest leave too few CTAs per SM).
static int vstat_band(const SepGrid &sg, int nmembers) {
    int BV = 16;
    while (BV < 256 && (long long)sg.ncx * ((sg.rhMax + 2 * BV - 1) / (2 * BV)) * nmembers >= 6 * 152) BV *= 2;
    return BV;
}

cudaError_t launch_sep_stats(const uint8_t *img, long long istride, int step, int iw, int ih, const MemberSet &ms,
                             int nmembers, int soloTw, int soloRw, const SepGrid &sg, int cnMin, int cnMax,
                             unsigned int *H, size_t slotStride, cudaStream_t st, int sharedPrefix,
                             cudaStream_t vst, cudaEvent_t vev, unsigned int *blk) {
    // a shared 4-channel prefix keeps its (s3, alpha squares) block after
    // the ih x hp x 4 main block (launch_row_prefix)
    HsumArgs h;
    h.img = img;
    h.istride = istride;
    h.step = step;
    h.iw = iw;
    h.ih = ih;
    h.rw = soloRw;
    h.tw = soloTw;
    h.hp = sg.hp;
    h.H = H;
    h.slotStride = slotStride;
    h.table = ms.table;
    h.first = ms.first;
    h.params = ms.params;
    h.pIdx = ms.solo.pIdx;
    VstatArgs v;
    v.H = H;
    v.slotStride = slotStride;
    v.alphaOff = (size_t)ih * sg.hp * 4;
    v.hp = sg.hp;
    v.ms = ms;
    v.BV = vstat_band(sg, nmembers);
    v.blk = nullptr;
    // One match: every band first sums th rows, so a tall template wants
    // tall bands (up to th / 2 rows, while ~8 warps per SM remain), and
    // narrower CTAs when the taller bands leave fewer than ~3 per SM.
    int VT = kThreads, ncx = sg.ncx;
    if (!sharedPrefix && !ms.table) {
        const long long warpCols = (soloRw + 31) / 32;
        int BV = 16;
        if (blk) {
            // the band starts from block sums: short bands, many of them
            v.blk = blk;
            BV = 32;
        } else {
            while (BV < 128 && 4 * BV <= ms.solo.th && warpCols * ((sg.rhMax + 2 * BV - 1) / (2 * BV)) >= 8 * 152)
                BV *= 2;
        }
        v.BV = BV;
        while (VT > 64 && (long long)((soloRw + VT - 1) / VT) * ((sg.rhMax + BV - 1) / BV) < 3 * 152) VT >>= 1;
        ncx = (soloRw + VT - 1) / VT;
    }
    const size_t smem = (size_t)(cnMax + 1) * (iw + 1) * sizeof(unsigned int);
    const int nb = (sg.rhMax + v.BV - 1) / v.BV;
    dim3 gh(ih, 1, nmembers), gv = sharedPrefix ? dim3(nmembers, sg.ncx, nb) : dim3(ncx, nb, nmembers);
    if (!sharedPrefix) {
        ProfScope ps("k_hsum", st);
        if (cnMax == 1) {
            set_smem(k_hsum<1, 1>, smem);
            k_hsum<1, 1><<<gh, kThreads, smem, st>>>(h);
        } else if (cnMax == 2) {
            set_smem(k_hsum<2, 2>, smem);
            k_hsum<2, 2><<<gh, kThreads, smem, st>>>(h);
        } else if (cnMin == 3) {
            set_smem(k_hsum<3, 4>, smem);
            k_hsum<3, 4><<<gh, kThreads, smem, st>>>(h);
        } else {
            set_smem(k_hsum<4, 4>, smem);
            k_hsum<4, 4><<<gh, kThreads, smem, st>>>(h);
        }
    }
    if (vst && vev) {
        // the vertical pass on its own stream, after the horizontal sums
        cudaError_t e = cudaEventRecord(vev, st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(vst, vev, 0);
        if (e != cudaSuccess) return e;
        st = vst;
    }
    if (sharedPrefix) v.blk = blk;  // a fleet's block sums, built once per frame (launch_vblock)
    if (v.blk && !sharedPrefix) {
        ProfScope ps("k_vblock", st);
        const size_t rowElems = (size_t)sg.hp * stat_pitch(cnMax);
        const int nblk = ih / 16;
        if (nblk > 0) {
            k_vblock<<<dim3((unsigned)((rowElems + kThreads - 1) / kThreads), nblk), kThreads, 0, st>>>(
                H, blk, nblk, rowElems);
            count_launches(1);
        }
    }
    {
        ProfScope ps("k_vstats", st);
        if (sharedPrefix && ms.form) {
            if (cnMax == 1)
                k_vstats<1, 1, true, true><<<gv, kThreads, 0, st>>>(v);
            else if (cnMax == 2)
                k_vstats<2, 2, true, true><<<gv, kThreads, 0, st>>>(v);
            else if (cnMin == 3)
                k_vstats<3, 4, true, true><<<gv, kThreads, 0, st>>>(v);
            else
                k_vstats<4, 4, true, true><<<gv, kThreads, 0, st>>>(v);
        } else if (ms.form) {
            if (cnMax == 1)
                k_vstats<1, 1, false, true><<<gv, VT, 0, st>>>(v);
            else if (cnMax == 2)
                k_vstats<2, 2, false, true><<<gv, VT, 0, st>>>(v);
            else if (cnMin == 3)
                k_vstats<3, 4, false, true><<<gv, VT, 0, st>>>(v);
            else
                k_vstats<4, 4, false, true><<<gv, VT, 0, st>>>(v);
        } else if (sharedPrefix) {
            if (cnMax == 1)
                k_vstats<1, 1, true><<<gv, kThreads, 0, st>>>(v);
            else if (cnMax == 2)
                k_vstats<2, 2, true><<<gv, kThreads, 0, st>>>(v);
            else if (cnMin == 3)
                k_vstats<3, 4, true><<<gv, kThreads, 0, st>>>(v);
            else
                k_vstats<4, 4, true><<<gv, kThreads, 0, st>>>(v);
        } else {
            if (cnMax == 1)
                k_vstats<1, 1, false><<<gv, VT, 0, st>>>(v);
            else if (cnMax == 2)
                k_vstats<2, 2, false><<<gv, VT, 0, st>>>(v);
            else if (cnMin == 3)
                k_vstats<3, 4, false><<<gv, VT, 0, st>>>(v);
            else
                k_vstats<4, 4, false><<<gv, VT, 0, st>>>(v);
        }
    }
    count_launches(sharedPrefix ? 1 : 2);
    return cudaGetLastError();
}

cudaError_t launch_vblock(const unsigned int *H, unsigned int *B, int nblk, size_t rowElems, cudaStream_t st) {
    if (nblk <= 0) return cudaSuccess;
    ProfScope ps("k_vblock", st);
    k_vblock<<<dim3((unsigned)((rowElems + kThreads - 1) / kThreads), nblk), kThreads, 0, st>>>(H, B, nblk, rowElems);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_sat(const unsigned int *P, int rows, size_t rowElems, unsigned int *B, unsigned int *S,
                       cudaStream_t st) {
    if (rows <= 0 || rowElems == 0) return cudaSuccess;
    const int nb = (rows + 15) / 16;
    const unsigned gx = (unsigned)((rowElems + kThreads - 1) / kThreads);
    ProfScope ps("k_sat", st);
    k_sat_blocks<<<dim3(gx, nb), kThreads, 0, st>>>(P, rows, rowElems, B);
    k_sat_scan<<<gx, kThreads, 0, st>>>(B, nb, rowElems);
    k_sat_fill<<<dim3(gx, nb + 1), kThreads, 0, st>>>(P, rows, rowElems, B, S);
    count_launches(3);
    return cudaGetLastError();
}

cudaError_t launch_row_prefix(const uint8_t *img, long long istride, int step, int iw, int ih, int cnP,
                              unsigned int *P, int hp, cudaStream_t st) {
    const int nq = cnP == 4 ? 6 : cnP + 1;
    const size_t smem = (size_t)nq * (iw + 1) * sizeof(unsigned int);
    const size_t ao = (size_t)ih * hp * 4;
    ProfScope ps("k_row_prefix", st);
    switch (cnP) {
        case 1: set_smem(k_row_prefix<1>, smem); k_row_prefix<1><<<ih, kThreads, smem, st>>>(img, istride, step, iw, P, hp, ao); break;
        case 2: set_smem(k_row_prefix<2>, smem); k_row_prefix<2><<<ih, kThreads, smem, st>>>(img, istride, step, iw, P, hp, ao); break;
        case 3: set_smem(k_row_prefix<3>, smem); k_row_prefix<3><<<ih, kThreads, smem, st>>>(img, istride, step, iw, P, hp, ao); break;
        default: set_smem(k_row_prefix<4>, smem); k_row_prefix<4><<<ih, kThreads, smem, st>>>(img, istride, step, iw, P, hp, ao); break;
    }
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_ingest(void *dst, size_t dpitch, const void *src, size_t spitch, size_t rowBytes, int rows,
                          cudaStream_t st) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | dpitch | spitch |
                        rowBytes;
    const int grid = 4 * 152;
    unsigned char *d = static_cast<unsigned char *>(dst);
    const unsigned char *s = static_cast<const unsigned char *>(src);
    ProfScope ps("k_ingest", st);
    if ((a & 15) == 0)
        k_ingest<uint4><<<grid, kThreads, 0, st>>>(d, dpitch, s, spitch, (int)(rowBytes / 16), rows);
    else if ((a & 3) == 0)
        k_ingest<unsigned int><<<grid, kThreads, 0, st>>>(d, dpitch, s, spitch, (int)(rowBytes / 4), rows);
    else
        k_ingest<unsigned char><<<grid, kThreads, 0, st>>>(d, dpitch, s, spitch, (int)rowBytes, rows);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t upload_bytes(void *dst, const void *src, size_t n, cudaStream_t st) {
    const unsigned char *p = static_cast<const unsigned char *>(src);
    unsigned char *d = static_cast<unsigned char *>(dst);
    while (n > 0) {
        UploadBlob b;
        const size_t c = n < sizeof(b.bytes) ? n : sizeof(b.bytes);
        for (size_t i = 0; i < c; i++) b.bytes[i] = p[i];
        {
            ProfScope ps("k_upload", st);
            k_upload<<<1, 256, 0, st>>>(d, b, (int)c);
        }
        count_launches(1);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        p += c;
        d += c;
        n -= c;
    }
    return cudaSuccess;
}

cudaError_t launch_shrink_gather(const float2 *src, int dftH, float2 *dst, int dh2, int hwp, int cnS,
                                 cudaStream_t st) {
    const long long total = (long long)cnS * dh2 * hwp;
    int blocks = (int)((total + kThreads - 1) / kThreads);
    if (blocks > 4096) blocks = 4096;
    ProfScope ps("k_shrink_gather", st);
    k_shrink_gather<<<blocks, kThreads, 0, st>>>(src, dftH, dst, dh2, hwp, cnS);
    count_launches(1);
    return cudaGetLastError();
}

void profile_enable(int on) {
    if (on) prof::collect();  // retire the records of an earlier window
    std::lock_guard<std::mutex> lk(prof::mu);
    prof::on = on != 0;
    if (on) {
        prof::totals.clear();
        prof::spans.clear();
        if (prof::origin) cudaEventDestroy(prof::origin);
        prof::origin = nullptr;
    }
}

int profile_span(int i, char *name, size_t len, double *t0, double *t1) {
    prof::collect();
    std::lock_guard<std::mutex> lk(prof::mu);
    if (i < 0 || i >= (int)prof::spans.size()) return 1;
    const prof::Span &sp = prof::spans[i];
    if (name && len) snprintf(name, len, "%s", sp.name.c_str());
    *t0 = sp.t0;
    *t1 = sp.t1;
    return 0;
}

int profile_read(int i, char *name, size_t len, double *ms, unsigned long long *count) {
    prof::collect();
    std::lock_guard<std::mutex> lk(prof::mu);
    if (i < 0 || i >= (int)prof::totals.size()) return 1;
    const prof::Total &t = prof::totals[i];
    if (name && len) {
        snprintf(name, len, "%s", t.name.c_str());
    }
    *ms = t.ms;
    *count = t.n;
    return 0;
}

}  // namespace cvm
