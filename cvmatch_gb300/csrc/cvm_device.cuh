// cvm_device.cuh -- device helpers shared by the kernel translation units
// (cvm_kernels.cu: the generic-size kernels; cvm_rows.cu: the row
// transforms specialised on the transform length).
//
// The butterfly and complex multiply are the reference's pinned op
// sequence (radix4.go:17-32, 80-149); every unit built on them keeps it.
#pragma once

#include <cfloat>
#include <climits>
#include <cstdint>

#include <cuda.h>

#include "cvm_internal.h"

namespace cvm {

namespace prof {
int begin(const char *name, cudaStream_t st);
void end(int idx, cudaStream_t st);
}  // namespace prof

// Programmatic dependent launch, device side.  griddep_wait: block until
// the kernel this one may overlap (the preceding kernel of its stream) has
// completed and its memory is visible -- a no-op when launched without
// the attribute.  griddep_launch: this CTA no longer holds back the
// launch of the stream's next kernel (which still waits before reading).
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// A transform kernel's launch, with the programmatic-serialization
// attribute when the calling thread asked for it (set_pdl); the kernel
// must call griddep_wait before its first global read.
template <typename... P, typename... A>
inline cudaError_t launch_k(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    if (pdl_on()) {
        at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        at[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, k, static_cast<A &&>(args)...);
}

// Brackets one launch with the optional per-kernel event timing.
struct ProfScope {
    int idx;
    cudaStream_t st;
    ProfScope(const char *name, cudaStream_t s) : idx(prof::begin(name, s)), st(s) {}
    ~ProfScope() { prof::end(idx, st); }
};

struct TileBox {
    int x0, y0, bw, bh, loadW, loadH;
};

struct Ext {
    float minV, maxV;
    long long minI, maxI;
};

struct InvArgs {
    TileGeom g;
    FftClass fc;
    int cls, cnS;
    MemberSet ms;
    int pairsPerCta;
    int partOffset;   // partial records of the classes before this one
    int nparts;       // partial records per member (all classes)
    Partial *partials;
    int *counters;    // per member params index
    cvm_result *out;
    const void *tcTab;  // the tensor-core kernel's tables (set by its launcher)
};

// Arguments of the column kernels (colsR4Go, mulConjGo; mode 0: forward
// spectrum, 1: forward + conj-multiply + inverse, 2: conj-multiply + inverse
// of a stored natural-order spectrum, 3: the fast form's channel sum of the
// conj-products + one inverse into channel slot 0).
struct ColsArgs {
    int mode;
    const float2 *in;
    float2 *out;
    int cnS;
    TileGeom g;
    FftClass fc;
    int cls;
    int chanCount;
    const int *cnDev;
    float scale;
    MemberSet ms;
    int SC, logSC;
    int nmem;   // members of the launch (waves: grid x = ntiles * nmem, z = strips)
};

// Arguments of the forward-rows kernels (forwardRowPair, impl.go:301-344).
struct FwdRowsArgs {
    const uint8_t *img;
    long long istride;
    int step, chanCount;
    const int *cnDev;        // device-side channel count (nullptr: chanCount)
    int chanFirst, chanGroup;
    TileGeom g;
    FftClass fc;
    float2 *spec;
    int cnS, pairsPerCta;
    int pix32;               // 4-byte pixels readable as aligned 32-bit words
    // each loaded sample is pixel * mul - sub[channel] (exact for the
    // integer values used: 1 and 0 for the reference's arithmetic, the
    // frame offset and the zero-mean template of the fast form); padding
    // stays zero
    float mul;
    float sub[4];
    // when set, sub[k] = subSums[k] / subDiv instead (template sums the
    // device computed; float, exact when subDiv == 1)
    const unsigned long long *subSums;
    float subDiv;
    int fma;                 // the fast form's samples: fused twiddle products
    // the fast form's zero-mean template without its sums on the device:
    // every CTA sums the template (this launch's one tile) itself, and
    // sub[k] = sum_k / subDiv
    int selfSums;
    // TMA staging of the CTA's frame rows (the tensor map passed beside the
    // arguments): boxes of 256 bytes x 2 pairsPerCta rows land at byte
    // offset tmaSmemOff of the dynamic shared memory, box i at
    // i * 256 * 2 pairsPerCta; 0 = plain loads
    int tma;
    unsigned int tmaSmemOff;
};

// The row transforms specialised on dftW = 2^5 .. 2^12 (cvm_rows.cu).
// map: the frame's tensor map when a.tma (ignored otherwise).
bool rows_fixed_length(int log2n);
// Elements (pairs x length) per CTA of a fleet wave's fast-form inverse rows.
int rows_fast_wave_elems(int log2n);
void launch_fwd_rows_fixed(const FwdRowsArgs &a, const CUtensorMap &map, dim3 grid, int threads, size_t smem,
                           cudaStream_t st);
// Encodes a 2-D tensor map over w x h bytes at img (row stride istride)
// with boxes of 256 bytes x boxRows rows; false when the driver entry point
// or the encoding is unavailable.
bool encode_frame_map(CUtensorMap *map, const void *img, long long istride, long long wBytes, int h, int boxRows);
// Sticky device flag of a TMA wait in the forward rows that gave up (read
// and cleared).
int rows_error_read_clear();
void launch_inv_rows_fixed(const InvArgs &a, dim3 grid, size_t smem, cudaStream_t st);
// The column kernels specialised on dftH = 2^5 .. 2^12 (cvm_cols.cu).
bool cols_fixed_length(int log2H);
void launch_cols_fixed(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st);
// Mode 4 (a colour match's fast form, fused channels): strip width for a
// height, and the launch (grid: strips x 1 x tiles).
int cols_sum_width(int log2H);
void launch_cols_sum(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st);

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int brev_bits(int x, int log2n) {
    return log2n == 0 ? 0 : (int)(__brev((unsigned)x) >> (32 - log2n));
}

// mulPlain (radix4.go:80-85): four single-rounded products, two sums.
__device__ __forceinline__ float2 cmul_plain(float2 v, float2 w) {
    float a = __fmul_rn(v.x, w.x), b = __fmul_rn(v.y, w.y);
    float c = __fmul_rn(v.x, w.y), d = __fmul_rn(v.y, w.x);
    return make_float2(__fsub_rn(a, b), __fadd_rn(c, d));
}

// The fast form's complex product: two products and two fused
// multiply-adds.
__device__ __forceinline__ float2 cmul_fma(float2 v, float2 w) {
    return make_float2(fmaf(v.x, w.x, -__fmul_rn(v.y, w.y)), fmaf(v.x, w.y, __fmul_rn(v.y, w.x)));
}

// One radix-4 butterfly (radix4.go:126-147); pa/pc/pb/pd are rows r, r+h,
// r+2h, r+3h.  The inverse conjugates the twiddles and flips the rotation.
// F (the fast form only): the twiddle products with fused multiply-adds.
template <bool INV, bool F = false>
__device__ __forceinline__ void bfly4(float2 *pa, float2 *pc, float2 *pb, float2 *pd, float2 bw,
                                      float2 cw, float2 dw) {
    if (INV) {
        bw.y = -bw.y;
        cw.y = -cw.y;
        dw.y = -dw.y;
    }
    const float2 av = *pa;
    const float2 tb = F ? cmul_fma(*pb, bw) : cmul_plain(*pb, bw);
    const float2 tc = F ? cmul_fma(*pc, cw) : cmul_plain(*pc, cw);
    const float2 td = F ? cmul_fma(*pd, dw) : cmul_plain(*pd, dw);
    if constexpr (F) {
        // the fast form's sums and differences on packed pairs: a - b as
        // fma(b, -1, a) rounds exactly as the subtraction does
        const float2 m1 = make_float2(-1.f, -1.f);
        const float2 s0 = __fadd2_rn(av, tc), s1 = __ffma2_rn(tc, m1, av);
        const float2 s2 = __fadd2_rn(tb, td), s3 = __ffma2_rn(td, m1, tb);
        const float rr = INV ? -s3.y : s3.y, ri = INV ? s3.x : -s3.x;
        *pa = __fadd2_rn(s0, s2);
        *pb = __ffma2_rn(s2, m1, s0);
        *pc = make_float2(__fadd_rn(s1.x, rr), __fadd_rn(s1.y, ri));
        *pd = make_float2(__fsub_rn(s1.x, rr), __fsub_rn(s1.y, ri));
        return;
    }
    const float s0x = __fadd_rn(av.x, tc.x), s0y = __fadd_rn(av.y, tc.y);
    const float s1x = __fsub_rn(av.x, tc.x), s1y = __fsub_rn(av.y, tc.y);
    const float s2x = __fadd_rn(tb.x, td.x), s2y = __fadd_rn(tb.y, td.y);
    const float s3x = __fsub_rn(tb.x, td.x), s3y = __fsub_rn(tb.y, td.y);
    float rr, ri;
    if (INV) {
        rr = -s3y;
        ri = s3x;
    } else {
        rr = s3y;
        ri = -s3x;
    }
    *pa = make_float2(__fadd_rn(s0x, s2x), __fadd_rn(s0y, s2y));
    *pc = make_float2(__fadd_rn(s1x, rr), __fadd_rn(s1y, ri));
    *pb = make_float2(__fsub_rn(s0x, s2x), __fsub_rn(s0y, s2y));
    *pd = make_float2(__fsub_rn(s1x, rr), __fsub_rn(s1y, ri));
}

// bfly4 with all three twiddles equal to 1 (quarter size 1, or column 0 of
// a stage): the fast form skips the products, which change nothing but the
// sign of a zero; the exact form keeps the reference's products.
template <bool INV>
__device__ __forceinline__ void bfly4_one(float2 *pa, float2 *pc, float2 *pb, float2 *pd) {
    const float2 av = *pa, tb = *pb, tc = *pc, td = *pd;
    {
        const float2 m1 = make_float2(-1.f, -1.f);
        const float2 s0 = __fadd2_rn(av, tc), s1 = __ffma2_rn(tc, m1, av);
        const float2 s2 = __fadd2_rn(tb, td), s3 = __ffma2_rn(td, m1, tb);
        const float rr = INV ? -s3.y : s3.y, ri = INV ? s3.x : -s3.x;
        *pa = __fadd2_rn(s0, s2);
        *pb = __ffma2_rn(s2, m1, s0);
        *pc = make_float2(__fadd_rn(s1.x, rr), __fadd_rn(s1.y, ri));
        *pd = make_float2(__fsub_rn(s1.x, rr), __fsub_rn(s1.y, ri));
        return;
    }
    const float s0x = av.x + tc.x, s0y = av.y + tc.y;
    const float s1x = av.x - tc.x, s1y = av.y - tc.y;
    const float s2x = tb.x + td.x, s2y = tb.y + td.y;
    const float s3x = tb.x - td.x, s3y = tb.y - td.y;
    const float rr = INV ? -s3y : s3y, ri = INV ? s3x : -s3x;
    *pa = make_float2(s0x + s2x, s0y + s2y);
    *pc = make_float2(s1x + rr, s1y + ri);
    *pb = make_float2(s0x - s2x, s0y - s2y);
    *pd = make_float2(s1x - rr, s1y - ri);
}

// normOne's score ladder (impl.go:825-849): |num| < den -> num / den,
// |num| < 1.125 den -> +-1, else 0.  The exact form divides correctly
// rounded, as the reference does.
__device__ __forceinline__ float score_exact(float num, float den) {
    const float an = fabsf(num);
    if (an < den) return __fdiv_rn(num, den);
    if (an < __fmul_rn(den, 1.125f)) return num > 0.f ? 1.f : -1.f;
    return 0.f;
}

// The fast form's ladder: the hardware division (within 2 ulp), except on
// near-flat windows, whose quotient num / den is formed in double precision
// and rounded once (a call on the rare path, so the epilogues keep their
// registers).  Near-flat: the window's variance (summed over its channels,
// from the exact integer sums) below one grey level squared, i.e.
// idiff < area^2, i.e. 0 < den < denFlat = sqrt(area) * templNorm -- a
// per-member constant (near_flat_den), so the test costs the epilogue one
// comparison and the statistics kernel nothing.
__device__ __noinline__ float score_near_flat(float num, float den) {
    const double d = (double)den, n = (double)num;
    if (fabs(n) < d) return __double2float_rn(__ddiv_rn(n, d));
    if (fabs(n) < d * 1.125) return num > 0.f ? 1.f : -1.f;
    return 0.f;
}

__device__ __forceinline__ float near_flat_den(int tw, int th, float templNorm) {
    return sqrtf((float)tw * (float)th) * templNorm;
}

__device__ __forceinline__ float score_fast(float num, float den, float denFlat) {
    const float an = fabsf(num);
    if (den > 0.f && den < denFlat) return score_near_flat(num, den);
    if (an < den) return __fdividef(num, den);
    if (an < den * 1.125f) return num > 0.f ? 1.f : -1.f;
    return 0.f;
}

// The fast form's den of the window at result (x, y) of member m, formed
// from the frame's summed-area table (MemberSet::sat) instead of read from
// the statistics kernel's lanes.  Four corners give the window's channel
// sums and its squared sum modulo 2^32; each channel sum is below 2^32,
// and the squared sum q is restored from its residue as
//   q = U - ((U - q) mod 2^32),   U = 255 * (sum of the channel sums),
// exact while U - q = sum over the window's bytes of v (255 - v), at most
// area * cn * 16256, stays below 2^32 (the host uses the table only
// then).  The rest is the statistics kernel's fast den sequence on the same
// integers (vstat_cols, FAST), so den has the same bits.
__device__ __forceinline__ float sat_den(const MemberSet &ms, const DevMember &m, const DevParams &Pm, int y, int x) {
    const size_t row = ms.satRow;
    unsigned int s0, s1 = 0u, s2 = 0u, s3 = 0u, qm;
    if (ms.satNp == 4) {
        const unsigned int *r0 = ms.sat + (size_t)y * row + (size_t)x * 4;
        const unsigned int *r1 = r0 + (size_t)m.th * row;
        const int dx = 4 * m.tw;
        const uint4 A = __ldg(reinterpret_cast<const uint4 *>(r1 + dx)), B = __ldg(reinterpret_cast<const uint4 *>(r1));
        const uint4 C = __ldg(reinterpret_cast<const uint4 *>(r0 + dx)), D = __ldg(reinterpret_cast<const uint4 *>(r0));
        s0 = A.x - B.x - C.x + D.x;
        s1 = A.y - B.y - C.y + D.y;
        s2 = A.z - B.z - C.z + D.z;
        qm = A.w - B.w - C.w + D.w;
        if (Pm.cn == 4) {
            // the (s3, alpha squares) block: half the main block's lanes per row
            const size_t arow = row >> 1;
            const unsigned int *a0 = ms.sat + ms.satAlpha + (size_t)y * arow + (size_t)x * 2;
            const unsigned int *a1 = a0 + (size_t)m.th * arow;
            const int da = 2 * m.tw;
            const uint2 A2 = __ldg(reinterpret_cast<const uint2 *>(a1 + da)), B2 = __ldg(reinterpret_cast<const uint2 *>(a1));
            const uint2 C2 = __ldg(reinterpret_cast<const uint2 *>(a0 + da)), D2 = __ldg(reinterpret_cast<const uint2 *>(a0));
            s3 = A2.x - B2.x - C2.x + D2.x;
            qm += A2.y - B2.y - C2.y + D2.y;
        }
    } else {
        const unsigned int *r0 = ms.sat + (size_t)y * row + (size_t)x * 2;
        const unsigned int *r1 = r0 + (size_t)m.th * row;
        const int dx = 2 * m.tw;
        const uint2 A = __ldg(reinterpret_cast<const uint2 *>(r1 + dx)), B = __ldg(reinterpret_cast<const uint2 *>(r1));
        const uint2 C = __ldg(reinterpret_cast<const uint2 *>(r0 + dx)), D = __ldg(reinterpret_cast<const uint2 *>(r0));
        s0 = A.x - B.x - C.x + D.x;
        qm = A.y - B.y - C.y + D.y;
    }
    const unsigned long long U = 255ull * ((unsigned long long)s0 + s1 + s2 + s3);
    const unsigned long long q = U - (unsigned int)((unsigned int)U - qm);
    const unsigned long long sq = (unsigned long long)s0 * s0 + (unsigned long long)s1 * s1 +
                                  (unsigned long long)s2 * s2 + (unsigned long long)s3 * s3;
    const unsigned long long idv = (unsigned long long)m.tw * m.th * q - sq;
    const float id = fmaf(__uint2float_rn((unsigned int)(idv >> 32)), 4294967296.0f, __uint2float_rn((unsigned int)idv));
    const float diff2 = __fmul_rn(id, Pm.varScale);
    float lim = 0.5f;
    if (q < (1ull << 24)) {
        lim = __fmul_rn(1.1920928955078125e-06f, __uint2float_rn((unsigned int)q));  // 10 * 2^-23 * q
        if (lim > 0.5f) lim = 0.5f;
    }
    const float sd = __fmul_rn(diff2, rsqrtf(diff2));
    return diff2 > lim ? __fmul_rn(sd, Pm.templNorm) : 0.f;
}

// Padded shared-memory line layout: one spare slot every 16 elements keeps
// the strided pass accesses free of bank conflicts.
__device__ __forceinline__ int padi(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int padded_len(int n) { return n + (n >> 4) + 1; }


__device__ __forceinline__ TileBox tile_box(const TileGeom &g, int tile) {
    TileBox b;
    const int tx = tile % g.ntx, ty = tile / g.ntx;
    b.x0 = tx * g.blockW;
    b.y0 = ty * g.blockH;
    b.bw = min(g.blockW, g.rwT - b.x0);
    b.bh = min(g.blockH, g.rhT - b.y0);
    b.loadW = b.bw + g.twL - 1;
    b.loadH = b.bh + g.thL - 1;
    return b;
}

__device__ __forceinline__ const DevMember &member_of(const MemberSet &ms, int slot) {
    return ms.table ? ms.table[ms.first + slot] : ms.solo;
}

// True when none of the tile's results lies in the member's region of
// interest (the member's own result extent cuts the last column/row).
__device__ __forceinline__ bool roi_misses_tile(const TileGeom &g, int tile, const TileBox &b, const DevMember &m) {
    const int ty = tile / g.ntx, tx = tile - ty * g.ntx;
    const int bw = (tx == g.ntx - 1) ? m.rw - b.x0 : g.blockW;
    const int bh = (ty == g.nty - 1) ? m.rh - b.y0 : g.blockH;
    return b.x0 >= m.roiX1 || b.x0 + bw <= m.roiX0 || b.y0 >= m.roiY1 || b.y0 + bh <= m.roiY0;
}

// ------------------------------------------------ first-occurrence extrema


__device__ __forceinline__ void ext_init(Ext &e) {
    e.minV = FLT_MAX;
    e.maxV = -FLT_MAX;
    e.minI = LLONG_MAX;
    e.maxI = LLONG_MAX;
}

// First occurrence in raster order with strict compares (impl.go:1023-1047,
// 1104-1112): a smaller value, or an equal value at a smaller index.
__device__ __forceinline__ void ext_add(Ext &e, float v, long long i) {
    if (v < e.minV || (v == e.minV && i < e.minI)) {
        e.minV = v;
        e.minI = i;
    }
    if (v > e.maxV || (v == e.maxV && i < e.maxI)) {
        e.maxV = v;
        e.maxI = i;
    }
}

// A thread that visits its results in increasing index order keeps the
// first occurrence with strict comparisons alone; ties between threads are
// broken by index when the partial extrema merge (ext_merge).
__device__ __forceinline__ void ext_add_inc(Ext &e, float v, long long i) {
    if (v < e.minV) {
        e.minV = v;
        e.minI = i;
    }
    if (v > e.maxV) {
        e.maxV = v;
        e.maxI = i;
    }
}

__device__ __forceinline__ void ext_merge(Ext &e, const Ext &o) {
    if (o.minV < e.minV || (o.minV == e.minV && o.minI < e.minI)) {
        e.minV = o.minV;
        e.minI = o.minI;
    }
    if (o.maxV > e.maxV || (o.maxV == e.maxV && o.maxI < e.maxI)) {
        e.maxV = o.maxV;
        e.maxI = o.maxI;
    }
}

__device__ void ext_block_reduce(Ext &e, Ext *sh) {
    for (int o = 16; o > 0; o >>= 1) {
        Ext t;
        t.minV = __shfl_down_sync(0xffffffffu, e.minV, o);
        t.maxV = __shfl_down_sync(0xffffffffu, e.maxV, o);
        t.minI = __shfl_down_sync(0xffffffffu, e.minI, o);
        t.maxI = __shfl_down_sync(0xffffffffu, e.maxI, o);
        ext_merge(e, t);
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sh[warp] = e;
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        if (lane < nw)
            e = sh[lane];
        else
            ext_init(e);
        for (int o = 16; o > 0; o >>= 1) {
            Ext t;
            t.minV = __shfl_down_sync(0xffffffffu, e.minV, o);
            t.maxV = __shfl_down_sync(0xffffffffu, e.maxV, o);
            t.minI = __shfl_down_sync(0xffffffffu, e.minI, o);
            t.maxI = __shfl_down_sync(0xffffffffu, e.maxI, o);
            ext_merge(e, t);
        }
    }
}

__device__ void ext_store_result(const Ext &e, int rw, cvm_result *out) {
    cvm_result r;
    if (e.minI == LLONG_MAX) {  // no result position (an empty region of interest)
        r.min_v = r.max_v = __int_as_float(0x7fc00000);
        r.min_x = r.min_y = r.max_x = r.max_y = -1;
        *out = r;
        return;
    }
    r.min_v = e.minV;
    r.max_v = e.maxV;
    r.min_x = (int32_t)(e.minI % rw);
    r.min_y = (int32_t)(e.minI / rw);
    r.max_x = (int32_t)(e.maxI % rw);
    r.max_y = (int32_t)(e.maxI / rw);
    *out = r;
}


__host__ __device__ constexpr int stat_pitch_c(int cn) { return stat_pitch(cn); }

// NP consecutive u32 (NP = 2, 4 or 8; 8- or 16-byte aligned) in one or two
// vector accesses.
template <int NP>
__device__ __forceinline__ void ldv(unsigned int *o, const unsigned int *p) {
    if constexpr (NP == 2) {
        const uint2 t = __ldg(reinterpret_cast<const uint2 *>(p));
        o[0] = t.x;
        o[1] = t.y;
    } else {
#pragma unroll
        for (int i = 0; i < NP; i += 4) {
            const uint4 t = __ldg(reinterpret_cast<const uint4 *>(p + i));
            o[i] = t.x;
            o[i + 1] = t.y;
            o[i + 2] = t.z;
            o[i + 3] = t.w;
        }
    }
}

template <int NP>
__device__ __forceinline__ void stv(unsigned int *p, const unsigned int *v) {
    if constexpr (NP == 2) {
        *reinterpret_cast<uint2 *>(p) = make_uint2(v[0], v[1]);
    } else {
#pragma unroll
        for (int i = 0; i < NP; i += 4) *reinterpret_cast<uint4 *>(p + i) = make_uint4(v[i], v[i + 1], v[i + 2], v[i + 3]);
    }
}

template <typename K>
void set_smem(K kernel, size_t bytes) {
    if (bytes > 48 * 1024)
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

}  // namespace
}  // namespace cvm
