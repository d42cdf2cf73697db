// cvm_tc.cu -- the mixed form's inverse row transforms on the tensor cores.
//
// The fast form's member tail inverts each tile's channel-summed spectrum
// row pair by row pair: the combine of inverseRowPair (impl.go:405-413)
// packs two spectrum rows into one complex 1024-point line z, whose
// inverse DFT x carries result row 2p in its real part and row 2p+1 in
// its imaginary part (impl.go:425-443); the FP32 form runs it as the
// radix-4 cascade (cvm_rows.cu).  Here the same inverse DFT runs as two
// dense 32-point DFT stages on the tensor cores (the four-step
// factorisation 1024 = 32 x 32):
//
//   k = 32 k1 + k2, n = n1 + 32 n2, w = e^{+2 pi i / 1024}, w32 = w^32
//   Y[n1, k2]        = sum_k1 z[32 k1 + k2] w32^(n1 k1)        (stage 1: MMA)
//   Y[n1, k2]       *= w^(n1 k2)                               (twiddle: FP32)
//   x[n1 + 32 n2]    = sum_k2 Y[n1, k2] w32^(n2 k2)            (stage 2: MMA)
//
// Each stage is one real GEMM D[128 x 64] = A[128 x 64] B[64 x 64] per four
// transforms: A's rows are (transform, k2) (stage 1) or (transform, n1)
// (stage 2) with K = 32 complex inputs as interleaved (re, im) pairs; B is
// the 32-point DFT matrix in real block form (out re = in re cos - in im
// sin, out im = in re sin + in im cos); D's 64 columns are the 32 complex
// outputs, interleaved the same way.  The products run as tcgen05.mma
// kind::f16 (FP16 operands, FP32 accumulation in TMEM) on split operands:
// each transform is first scaled by the power of two that brings its
// largest magnitude just below 2^14 (FP16's range), then every operand is
// split as hi = fp16(v), lo = fp16(v - hi), and the products are
// accumulated as Ahi Bhi + Alo Bhi + Ahi Blo: ~22 significant bits per
// operand, the FP32 cascade's order of error.  The stage-2 operand keeps
// that scale times 2^-6 (a 32-point stage grows magnitudes by less than
// 2^6), and the scale is undone (exactly, a power of two) when D is read
// back.  One thread issues the MMAs;
// tcgen05.commit arrives on an mbarrier the CTA waits on (a bounded wait:
// after ~2 s without the arrival it records a device error, frees its TMEM
// and returns); D comes back from TMEM with tcgen05.ld.  Operands are staged
// in shared memory in the K-major, no-swizzle core-matrix layout (8 rows x
// 16 bytes per core matrix), A with a 144-byte K stride so the transposed
// stores between the stages are free of bank conflicts; the DFT matrix and
// the twiddles are built once per device in double precision.
//
// The epilogue is the FP32 kernel's: normOne's ladder from the den lanes
// of the statistics kernel, first-occurrence extrema, the member's result
// from its last CTA.  Scores differ from the FP32 fast form by rounding.
#include <cuda_fp16.h>

#include <cmath>
#include <cstdio>
#include <mutex>
#include <vector>

#include "cvm_device.cuh"

namespace cvm {
namespace {

constexpr int kTcThreads = 128;  // one warpgroup: warp w owns TMEM lanes 32w..32w+31
constexpr int kTcM = 128;        // MMA rows: 4 transforms x 32
constexpr int kTcTrans = 4;      // transforms per MMA tile
constexpr uint32_t kTcCols = 64; // TMEM columns: D is 128 lanes x 64 fp32
// Operand layouts (bytes, fp16 elements).  Core matrix (row group g, K
// chunk c of 8 halves) at g * SBO + c * LBO; row r % 8 at +16 (r % 8),
// element k % 8 at +2 (k % 8).
constexpr uint32_t A_LBO = 144, A_SBO = 8 * A_LBO, A_BYTES = (kTcM / 8) * A_SBO;   // 18432
constexpr uint32_t B_LBO = 128, B_SBO = 8 * B_LBO, B_BYTES = (64 / 8) * B_SBO;     // 8192
constexpr uint32_t OFF_AHI = 0, OFF_ALO = A_BYTES, OFF_BHI = 2 * A_BYTES, OFF_BLO = 2 * A_BYTES + B_BYTES;
constexpr uint32_t TC_SMEM = 2 * A_BYTES + 2 * B_BYTES;    // 53248: four CTAs per SM
constexpr size_t kTcSmemLaunch = TC_SMEM + 1024;           // + alignment slack
// Per-transform scaling: operands are multiplied by a power of two that
// puts the transform's largest magnitude just below 2^14 (FP16's range
// ends at 65504; K = 64 sums of products of magnitude <= 2^14 stay in FP32).
constexpr int kTcScaleExp = 14;

// The 32-point DFT matrix in real block form (B[n][k]: out re/im n, in
// re/im k) as the shared-memory image of its FP16 hi and lo halves, and
// the 1024 twiddles w^j = (cos, sin)(2 pi j / 1024); built once per device
// from double precision.
struct TcTables {
    unsigned char bimg[2 * B_BYTES];
    float2 tw[1024];
};

__device__ int g_tc_error = 0;  // a tensor-core wait that gave up (sticky until read and cleared)

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__host__ __device__ __forceinline__ uint32_t a_off(int row, int k) {
    return (uint32_t)(row >> 3) * A_SBO + (uint32_t)(k >> 3) * A_LBO + (uint32_t)(row & 7) * 16u + (uint32_t)(k & 7) * 2u;
}
__host__ __device__ __forceinline__ uint32_t b_off(int n, int k) {
    return (uint32_t)(n >> 3) * B_SBO + (uint32_t)(k >> 3) * B_LBO + (uint32_t)(n & 7) * 16u + (uint32_t)(k & 7) * 2u;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (row-group) byte offsets, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: D f32 (bits 4-5 = 1), A and B f16
// (bits 7-9, 10-12 = 0), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kIdesc = (1u << 4) | ((64u >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, int accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %3, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %4, p;\n\t}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(accum), "r"(kIdesc));
}

__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try(uint32_t addr, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.b32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(addr), "r"(phase)
        : "memory");
    return ok != 0;
}

// Waits for the mbarrier phase; gives up after ~2^32 cycles (about 2 s),
// recording the failure in g_tc_error.
__device__ __noinline__ bool mbar_wait(uint64_t *bar, uint32_t phase) {
    const uint32_t addr = smem_u32(bar);
    const long long t0 = clock64();
    for (unsigned it = 0;; it++) {
        if (mbar_try(addr, phase)) return true;
        if ((it & 255u) == 255u && clock64() - t0 > (1ll << 32)) {
            atomicExch(&g_tc_error, 1);
            return false;
        }
    }
}

// 32 consecutive TMEM columns of this warp's 32 lanes, one lane per thread.
// The load and its wait are one asm statement, so no use of the registers
// can be scheduled before the data has arrived.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive TMEM columns (the same contract as tmem_ld32).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// The power of two that scales a transform whose largest magnitude is m
// to just below 2^kTcScaleExp (1 for an all-zero transform), and its inverse.
__device__ __forceinline__ float2 tc_scale(float m) {
    if (!(m > 0.f)) return make_float2(1.f, 1.f);
    int e;
    frexpf(m, &e);  // m = f 2^e, f in [0.5, 1)
    return make_float2(ldexpf(1.f, kTcScaleExp - e), ldexpf(1.f, e - kTcScaleExp));
}

__device__ __forceinline__ float warp_max(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// hi = fp16(v), lo = fp16(v - hi): the two halves of a split operand.
__device__ __forceinline__ void split2(float v, __half &hi, __half &lo) {
    hi = __float2half_rn(v);
    lo = __float2half_rn(v - __half2float(hi));
}

// The CTA's tensor-core state: TMEM columns, the MMA-completion mbarrier
// and its phase.
struct TcState {
    uint32_t tmem;
    uint32_t phase;
    bool ok;
};

// Copies B (hi, lo) into shared memory, allocates TMEM (warp 0) and
// initialises the mbarrier.
__device__ void tc_setup(unsigned char *sm, const TcTables *__restrict__ tab, uint64_t *bar, uint32_t *tmemSlot,
                         TcState &s) {
    const int tid = threadIdx.x;
    const uint4 *src = reinterpret_cast<const uint4 *>(tab->bimg);
    uint4 *dst = reinterpret_cast<uint4 *>(sm + OFF_BHI);
    for (int i = tid; i < (int)(2 * B_BYTES / 16); i += blockDim.x) dst[i] = __ldg(src + i);
    if (tid < 32) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmemSlot)),
                     "r"(kTcCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    s.tmem = *tmemSlot;
    s.phase = 0;
    s.ok = true;
}

__device__ void tc_teardown(const TcState &s) {
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (threadIdx.x < 32) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(s.tmem), "r"(kTcCols));
}

// hi/lo halves of two values at once (packed conversions).
__device__ __forceinline__ void split_pair(float a, float b, __half2 &hi, __half2 &lo) {
    hi = __floats2half2_rn(a, b);
    const float2 h = __half22float2(hi);
    lo = __floats2half2_rn(a - h.x, b - h.y);
}

// Stage-1 operand: this thread's row (32 warp + lane) from its 32 complex
// inputs z[k1] = (re[k1], im[k1]) at K = 2 k1 (re), 2 k1 + 1 (im), scaled
// by sc and split; one 16-byte store per chunk of 4 complex values.
__device__ __forceinline__ void a_store_row(unsigned char *sm, int row, const float *re, const float *im, float sc) {
#pragma unroll
    for (int c = 0; c < 8; c++) {
        __align__(16) __half2 h[4], l[4];
#pragma unroll
        for (int i = 0; i < 4; i++) split_pair(re[4 * c + i] * sc, im[4 * c + i] * sc, h[i], l[i]);
        const uint32_t o = a_off(row, 8 * c);
        *reinterpret_cast<uint4 *>(sm + OFF_AHI + o) = *reinterpret_cast<const uint4 *>(h);
        *reinterpret_cast<uint4 *>(sm + OFF_ALO + o) = *reinterpret_cast<const uint4 *>(l);
    }
}

// One stage: D = Ahi Bhi + Alo Bhi + Ahi Blo over K = 64 (4 steps of 16),
// issued by thread 0, completion on the mbarrier; every thread then waits.
// The caller has stored A (fence.proxy.async by every writer) and
// synchronised.
__device__ void tc_stage(unsigned char *sm, uint64_t *bar, TcState &s) {
    if (threadIdx.x == 0 && s.ok) {
        tc_fence_after();
        const uint32_t base = smem_u32(sm);
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {
            const uint64_t ah = sdesc(base + OFF_AHI + ks * 2 * A_LBO, A_LBO, A_SBO);
            const uint64_t al = sdesc(base + OFF_ALO + ks * 2 * A_LBO, A_LBO, A_SBO);
            const uint64_t bh = sdesc(base + OFF_BHI + ks * 2 * B_LBO, B_LBO, B_SBO);
            const uint64_t bl = sdesc(base + OFF_BLO + ks * 2 * B_LBO, B_LBO, B_SBO);
            mma_f16(s.tmem, ah, bh, ks > 0);
            mma_f16(s.tmem, al, bh, 1);
            mma_f16(s.tmem, ah, bl, 1);
        }
        tc_commit(bar);
    }
    if (s.ok) s.ok = mbar_wait(bar, s.phase);
    s.phase ^= 1;
    tc_fence_after();
}

// After stage 1: thread (warp w, lane k2) reads D[., k2] of transform w
// (= Y scaled by sc1, columns (re, im) of n1 at 2 n1, 2 n1 + 1), applies
// the twiddles w^(n1 k2) and stores the stage-2 operand: row 32 w + n1,
// K = 2 k2 (re) and 2 k2 + 1 (im), one 4-byte store each for hi and lo.
// The stage-2 operand is Y w^(n1 k2) scaled by sc1 2^-6: the twiddles have
// unit modulus and a 32-point stage grows magnitudes by at most 32 sqrt(2)
// < 2^6, so it stays below 2^14 as stage 1's did, with no second search
// for the maximum; 32 columns at a time.
__device__ void tc_twiddle_transpose(unsigned char *sm, const TcTables *__restrict__ tab, const TcState &s) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t ta = s.tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
    for (int hf = 0; hf < 2; hf++) {
        float y[32];
        tmem_ld32(ta + 32 * hf, y);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            const int n1 = 16 * hf + j;
            float2 w = __ldg(tab->tw + n1 * lane);
            w.x *= 0.015625f;  // 2^-6
            w.y *= 0.015625f;
            const float yr = y[2 * j], yi = y[2 * j + 1];
            __half2 h, l;
            split_pair(fmaf(yr, w.x, -yi * w.y), fmaf(yr, w.y, yi * w.x), h, l);
            const uint32_t o = a_off(32 * warp + n1, 2 * lane);
            *reinterpret_cast<__half2 *>(sm + OFF_AHI + o) = h;
            *reinterpret_cast<__half2 *>(sm + OFF_ALO + o) = l;
        }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
}

// ------------------------------------------------------------ self-test

// Four inverse 1024-point DFTs of z (natural order, complex) into x, and
// the first stage's GEMM tile, unscaled, into d1 (128 x 64).
__global__ void __launch_bounds__(kTcThreads, 1) k_tc_selftest(const TcTables *__restrict__ tab,
                                                              const float2 *__restrict__ z, float2 *__restrict__ x,
                                                              float *__restrict__ d1) {
    extern __shared__ unsigned char smraw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmemSlot;
    TcState s;
    tc_setup(sm, tab, &bar, &tmemSlot, s);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float re[32], im[32], m = 0.f;
#pragma unroll
    for (int k1 = 0; k1 < 32; k1++) {
        const float2 e = z[warp * 1024 + 32 * k1 + lane];
        re[k1] = e.x;
        im[k1] = e.y;
        m = fmaxf(m, fmaxf(fabsf(e.x), fabsf(e.y)));
    }
    const float2 sc1 = tc_scale(warp_max(m));
    a_store_row(sm, 32 * warp + lane, re, im, sc1.x);
    fence_async_smem();
    __syncthreads();
    tc_stage(sm, &bar, s);
    {
        // stored as (re[32], im[32]) per row
        float v[32];
        const uint32_t ta = s.tmem + ((uint32_t)(32 * warp) << 16);
        tmem_ld32(ta, v);
#pragma unroll
        for (int i = 0; i < 16; i++) {
            d1[(32 * warp + lane) * 64 + i] = v[2 * i] * sc1.y;
            d1[(32 * warp + lane) * 64 + 32 + i] = v[2 * i + 1] * sc1.y;
        }
        tmem_ld32(ta + 32, v);
#pragma unroll
        for (int i = 0; i < 16; i++) {
            d1[(32 * warp + lane) * 64 + 16 + i] = v[2 * i] * sc1.y;
            d1[(32 * warp + lane) * 64 + 48 + i] = v[2 * i + 1] * sc1.y;
        }
    }
    tc_twiddle_transpose(sm, tab, s);
    const float inv2 = sc1.y * 64.f;  // the stage-2 operand was scaled by sc1 2^-6
    tc_stage(sm, &bar, s);
    float v[32];
    const uint32_t ta = s.tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll
    for (int hf = 0; hf < 2; hf++) {
        tmem_ld32(ta + 32 * hf, v);
#pragma unroll
        for (int i = 0; i < 16; i++)
            x[warp * 1024 + lane + 32 * (16 * hf + i)] = make_float2(v[2 * i] * inv2, v[2 * i + 1] * inv2);
    }
    tc_teardown(s);
}

// --------------------------------------------------------- inverse rows

// The fast form's fused inverse rows (k_inv_rows_t<10, true> with the
// radix-4 cascade replaced): four row pairs per MMA tile, pairsPerCta row
// pairs per CTA (the same grid and partial records as the FP32 kernel).
__global__ void __launch_bounds__(kTcThreads, 4) k_inv_rows_tc(InvArgs a) {
    griddep_wait();
    constexpr int N = 1024, HALF = 512;
    extern __shared__ unsigned char smraw[];
    unsigned char *sm = reinterpret_cast<unsigned char *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023));
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmemSlot;
    __shared__ Ext shExt[kTcThreads / 32];
    __shared__ int isLast;
    const TcTables *tab = reinterpret_cast<const TcTables *>(a.tcTab);
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
    int P = 2 * pair0 < bh ? min(a.pairsPerCta, (bh - 2 * pair0 + 1) >> 1) : 0;
    if (P > 0 && a.ms.anyRoi) {
        const int ya = tb.y0 + 2 * pair0, yb = tb.y0 + min(2 * (pair0 + P), bh);
        if (ya >= m.roiY1 || yb <= m.roiY0 || tb.x0 >= m.roiX1 || tb.x0 + bw <= m.roiX0) P = 0;
    }
    const bool flat = Pm.flat != 0;
    const float denFlat = near_flat_den(m.tw, m.th, Pm.templNorm);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int log2H = fc.log2H, hwp = fc.hwp;
    const float2 *cb = a.ms.scratch[a.cls] + (size_t)slot * a.ms.scratchStride[a.cls] +
                       (size_t)tileLocal * a.cnS * fc.dftH * hwp;
    const float *dens = reinterpret_cast<const float *>(a.ms.lanes + (size_t)slot * a.ms.lanesStride);
    float *map = a.ms.map;
    const int xlo = m.roiX0 - tb.x0, xhi = m.roiX1 - tb.x0;
    Ext e;
    ext_init(e);
    if (flat) {
        // a flat template scores 1 everywhere (impl.go:1137-1144)
        for (int rr = 0; rr < 2 * P; rr++) {
            const int r = 2 * pair0 + rr;
            if (r >= bh) break;
            const long long rowBase = (long long)(tb.y0 + r) * m.rw + tb.x0;
            for (int x = threadIdx.x; x < bw; x += kTcThreads) {
                if (map) map[rowBase + x] = 1.f;
                if (x >= xlo && x < xhi) ext_add_inc(e, 1.f, rowBase + x);
            }
        }
    } else if (P > 0) {
        TcState s;
        tc_setup(sm, tab, &bar, &tmemSlot, s);
        for (int t0 = 0; t0 < P; t0 += kTcTrans) {
            // stage-1 operand from the combine (impl.go:405-413): thread
            // (w, k2) builds row 32 w + k2 = z[32 k1 + k2], k1 = 0..31, of
            // row pair t0 + w
            const int p = t0 + warp;
            const bool live = p < P;
            const int r = 2 * (pair0 + p);
            float re[32], im[32], mx = 0.f;
            {
                const float2 *u = cb + (size_t)brev_bits(live ? r : 0, log2H) * hwp;
                const float2 *v = cb + (size_t)brev_bits(live ? r + 1 : 0, log2H) * hwp;
#pragma unroll
                for (int k1 = 0; k1 < 32; k1++) {
                    const int k = 32 * k1 + lane;
                    float2 U = make_float2(0.f, 0.f), V = U;
                    if (live) {
                        const int kk = k <= HALF ? k : N - k;
                        U = __ldg(u + kk);
                        V = __ldg(v + kk);
                    }
                    if (k <= HALF) {
                        re[k1] = U.x - V.y;
                        im[k1] = U.y + V.x;
                    } else {
                        re[k1] = U.x + V.y;
                        im[k1] = V.x - U.y;
                    }
                    mx = fmaxf(mx, fmaxf(fabsf(re[k1]), fabsf(im[k1])));
                }
            }
            const float2 sc1 = tc_scale(warp_max(mx));
            a_store_row(sm, 32 * warp + lane, re, im, sc1.x);
            fence_async_smem();
            __syncthreads();
            tc_stage(sm, &bar, s);
            tc_twiddle_transpose(sm, tab, s);
            const float inv2 = sc1.y * 64.f;  // the stage-2 operand was scaled by sc1 2^-6
            tc_stage(sm, &bar, s);
            // x[lane + 32 n2] = (re, im) at columns 2 n2, 2 n2 + 1: re is
            // result row r, im row r + 1; 16 values of n2 per TMEM read, den
            // first (their loads overlap the TMEM read).  The two rows'
            // results interleave, so the extrema break ties by index
            // explicitly (ext_add).
            const uint32_t ta = s.tmem + ((uint32_t)(32 * warp) << 16);
            const long long rowBase0 = (long long)(tb.y0 + r) * m.rw + tb.x0, rowBase1 = rowBase0 + m.rw;
            const bool on0 = live && r < bh && tb.y0 + r >= m.roiY0 && tb.y0 + r < m.roiY1;
            const bool on1 = live && r + 1 < bh && tb.y0 + r + 1 >= m.roiY0 && tb.y0 + r + 1 < m.roiY1;
#pragma unroll 1
            for (int q = 0; q < 4; q++) {
                // results x = lane + 32 n2, n2 = 8 q .. 8 q + 7 (TMEM columns 16 q ..)
                float d0[8], d1[8];
#pragma unroll
                for (int i = 0; i < 8; i++) {
                    const int x = lane + 32 * (8 * q + i);
                    d0[i] = (on0 && x < bw) ? __ldg(dens + rowBase0 + x) : 0.f;
                    d1[i] = (on1 && x < bw) ? __ldg(dens + rowBase1 + x) : 0.f;
                }
                float xv[16];
                tmem_ld16(ta + 16 * q, xv);
                if (s.ok) {
#pragma unroll
                    for (int i = 0; i < 8; i++) {
                        const int x = lane + 32 * (8 * q + i);
                        if (x < bw) {
                            const bool inx = x >= xlo && x < xhi;
                            if (on0) {
                                const float score = score_fast(xv[2 * i] * inv2, d0[i], denFlat);
                                if (map) map[rowBase0 + x] = score;
                                if (inx) ext_add(e, score, rowBase0 + x);
                            }
                            if (on1) {
                                const float score = score_fast(xv[2 * i + 1] * inv2, d1[i], denFlat);
                                if (map) map[rowBase1 + x] = score;
                                if (inx) ext_add(e, score, rowBase1 + x);
                            }
                        }
                    }
                }
            }
            // the next tile's stores overwrite A and its MMAs D
            tc_fence_before();
            __syncthreads();
            tc_fence_after();
        }
        tc_teardown(s);
    }
    __syncthreads();
    ext_block_reduce(e, shExt);
    if (threadIdx.x == 0) {
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
    for (int i = threadIdx.x; i < a.nparts; i += kTcThreads) {
        const volatile Partial *pp = a.partials + m.partBase + i;
        Ext o;
        o.minV = pp->minV;
        o.maxV = pp->maxV;
        o.minI = pp->minI;
        o.maxI = pp->maxI;
        ext_merge(e, o);
    }
    __syncthreads();
    ext_block_reduce(e, shExt);
    if (threadIdx.x == 0) ext_store_result(e, m.rw, a.out + m.outIdx);
}

TcTables *g_tab = nullptr;  // device copy, built by tc_init

}  // namespace

// Builds the device tables once (called from the library's device set-up).
cudaError_t tc_init() {
    if (g_tab) return cudaSuccess;
    std::vector<unsigned char> img(sizeof(TcTables), 0);
    TcTables *h = reinterpret_cast<TcTables *>(img.data());
    const double PI2 = 6.283185307179586476925286766559;
    // B[n][k]: output n = 2 n1 + (0 re, 1 im), input k = 2 k1 + (0 re, 1 im)
    for (int n = 0; n < 64; n++)
        for (int k = 0; k < 64; k++) {
            const int n1 = n >> 1, k1 = k >> 1, on = n & 1, ik = k & 1;
            const double th = PI2 * (double)((n1 * k1) & 31) / 32.0, c = std::cos(th), sn = std::sin(th);
            const double v = on == 0 ? (ik == 0 ? c : -sn) : (ik == 0 ? sn : c);
            const float vf = (float)v;
            const __half hi = __float2half_rn(vf), lo = __float2half_rn(vf - __half2float(hi));
            *reinterpret_cast<__half *>(h->bimg + b_off(n, k)) = hi;
            *reinterpret_cast<__half *>(h->bimg + B_BYTES + b_off(n, k)) = lo;
        }
    for (int j = 0; j < 1024; j++) {
        const double th = PI2 * j / 1024.0;
        h->tw[j] = make_float2((float)std::cos(th), (float)std::sin(th));
    }
    TcTables *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(TcTables));
    if (e == cudaSuccess) e = cudaMemcpy(d, img.data(), sizeof(TcTables), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        if (d) cudaFree(d);
        return e;
    }
    g_tab = d;
    return cudaSuccess;
}

bool inv_rows_tc_applies(const FftClass &fc, const MemberSet &ms) {
    return ms.form == CVM_FORM_MIXED && fc.log2n == 10 && ms.lanes != nullptr && g_tab != nullptr;
}

cudaError_t launch_inv_rows_tc(const InvArgs &a, dim3 grid, cudaStream_t st) {
    InvArgs b = a;
    b.tcTab = g_tab;
    set_smem(k_inv_rows_tc, kTcSmemLaunch);
    return launch_k(k_inv_rows_tc, grid, dim3(kTcThreads), kTcSmemLaunch, st, b);
}

int tc_error_read_clear() {
    int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof v) != cudaSuccess) return -1;
    if (v) cudaMemcpyToSymbol(g_tc_error, &z, sizeof z);
    return v;
}

// Runs the self-test kernel on four pseudo-random lines and compares with
// the DFT in double precision; returns the largest errors relative to each
// line's norm (whole DFT; first stage alone), or a CUDA error.
cudaError_t tc_selftest(double *dftErr, double *gemmErr) {
    cudaError_t e = tc_init();
    if (e != cudaSuccess) return e;
    const int T = 4, N = 1024;
    std::vector<float2> z(T * N);
    uint32_t st = 12345u;
    for (auto &c : z) {
        st = st * 1664525u + 1013904223u;
        c.x = (float)((int)(st >> 8) % 2001 - 1000) * 0.37f;
        st = st * 1664525u + 1013904223u;
        c.y = (float)((int)(st >> 8) % 2001 - 1000) * 0.37f;
    }
    float2 *dz = nullptr, *dx = nullptr;
    float *dd = nullptr;
    e = cudaMalloc(&dz, T * N * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&dx, T * N * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&dd, 128 * 64 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(dz, z.data(), T * N * sizeof(float2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmemLaunch);
    if (e == cudaSuccess) {
        k_tc_selftest<<<1, kTcThreads, kTcSmemLaunch>>>(g_tab, dz, dx, dd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    std::vector<float2> x(T * N);
    std::vector<float> d(128 * 64);
    if (e == cudaSuccess) e = cudaMemcpy(x.data(), dx, T * N * sizeof(float2), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(d.data(), dd, 128 * 64 * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(dz);
    cudaFree(dx);
    cudaFree(dd);
    if (e != cudaSuccess) return e;
    const double PI2 = 6.283185307179586476925286766559;
    double worstX = 0, worstD = 0;
    for (int t = 0; t < T; t++) {
        double norm = 0;
        for (int k = 0; k < N; k++) norm += (double)z[t * N + k].x * z[t * N + k].x + (double)z[t * N + k].y * z[t * N + k].y;
        norm = std::sqrt(norm);
        for (int n = 0; n < N; n++) {
            double re = 0, im = 0;
            for (int k = 0; k < N; k++) {
                const double th = PI2 * (double)((long long)n * k % N) / N, c = std::cos(th), s = std::sin(th);
                re += z[t * N + k].x * c - z[t * N + k].y * s;
                im += z[t * N + k].x * s + z[t * N + k].y * c;
            }
            const double err = std::hypot(x[t * N + n].x - re, x[t * N + n].y - im) / norm;
            if (err > worstX) worstX = err;
        }
        // stage 1 alone: D[32 t + k2][n] for the 32-point DFTs over k1
        for (int k2 = 0; k2 < 32; k2++) {
            double n1norm = 0;
            for (int k1 = 0; k1 < 32; k1++) {
                const float2 c = z[t * N + 32 * k1 + k2];
                n1norm += (double)c.x * c.x + (double)c.y * c.y;
            }
            n1norm = std::sqrt(n1norm) + 1e-30;
            for (int n1 = 0; n1 < 32; n1++) {
                double re = 0, im = 0;
                for (int k1 = 0; k1 < 32; k1++) {
                    const float2 c = z[t * N + 32 * k1 + k2];
                    const double th = PI2 * (double)((n1 * k1) % 32) / 32, cs = std::cos(th), sn = std::sin(th);
                    re += c.x * cs - c.y * sn;
                    im += c.x * sn + c.y * cs;
                }
                const float *row = &d[(32 * t + k2) * 64];
                const double err = std::hypot(row[n1] - re, row[32 + n1] - im) / n1norm;
                if (err > worstD) worstD = err;
            }
        }
    }
    *dftErr = worstX;
    *gemmErr = worstD;
    return cudaSuccess;
}

}  // namespace cvm
