// cvm_rows.cu -- the row transforms specialised on the transform length.
//
// forwardRowPair (impl.go:301-344) and inverseRowPair (impl.go:394-444)
// for dftW = 2^5 .. 2^12, one kernel instance per length.  The arithmetic
// is exactly that of the generic-length kernels in cvm_kernels.cu (same
// butterflies, same twiddles, same order of every rounded op); what the
// fixed length buys is addressing: with the length and each pass's
// quarter size known at compile time, every element of a radix unit sits
// at a constant offset from the unit's first element in the padded
// shared-memory line, so a unit costs one address computation instead of
// one per element.  Other lengths run the generic kernels.
#include <cudaTypedefs.h>

#include "cvm_device.cuh"

namespace cvm {
namespace {

// padi() of a compile-time index.
__host__ __device__ constexpr int padc(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v >> 1); }

template <int LOG2N>
__device__ __forceinline__ int brevn(int x) {
    return (int)(__brev((unsigned)x) >> (32 - LOG2N));
}

// Element i of a unit of quarter size H starting at base = blk*R*H + j
// (j < H) sits at padi(base) + padc(H*i): for H >= 16 the pad counter is
// linear in i, and for H < 16 the low bits j + (H*i mod 16) never reach 16.
template <bool INV, int H, bool F = false>
__device__ __forceinline__ void unit16(float2 *p, const float2 *__restrict__ tA, const float2 *__restrict__ tB) {
    float2 e[16];
#pragma unroll
    for (int i = 0; i < 16; i++) e[i] = p[padc(H * i)];
    if constexpr (F && H == 1) {
        // quarter 1: the first stage's twiddles and the second stage's
        // column 0 are all 1
#pragma unroll
        for (int b = 0; b < 4; b++) bfly4_one<INV>(&e[4 * b], &e[4 * b + 1], &e[4 * b + 2], &e[4 * b + 3]);
        bfly4_one<INV>(&e[0], &e[4], &e[8], &e[12]);
#pragma unroll
        for (int q = 1; q < 4; q++)
            bfly4<INV, F>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + q), __ldg(tB + 4 + q),
                          __ldg(tB + 8 + q));
    } else {
        const float2 a1 = __ldg(tA), a2 = __ldg(tA + H), a3 = __ldg(tA + 2 * H);
#pragma unroll
        for (int b = 0; b < 4; b++)
            bfly4<INV, F>(&e[4 * b], &e[4 * b + 1], &e[4 * b + 2], &e[4 * b + 3], a1, a2, a3);
#pragma unroll
        for (int q = 0; q < 4; q++)
            bfly4<INV, F>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + H * q), __ldg(tB + 4 * H + H * q),
                          __ldg(tB + 8 * H + H * q));
    }
#pragma unroll
    for (int i = 0; i < 16; i++) p[padc(H * i)] = e[i];
}

template <bool INV, int H, bool F = false>
__device__ __forceinline__ void unit4(float2 *p, const float2 *__restrict__ t) {
    float2 e[4];
#pragma unroll
    for (int i = 0; i < 4; i++) e[i] = p[padc(H * i)];
    bfly4<INV, F>(&e[0], &e[1], &e[2], &e[3], __ldg(t), __ldg(t + H), __ldg(t + 2 * H));
#pragma unroll
    for (int i = 0; i < 4; i++) p[padc(H * i)] = e[i];
}

// The radix-2 head and the h=2 stage on 8 contiguous elements.
template <bool INV, bool F = false>
__device__ __forceinline__ void unit_head(float2 *p, const float2 *__restrict__ t) {
    float2 e[8];
#pragma unroll
    for (int i = 0; i < 8; i++) e[i] = p[i];
#pragma unroll
    for (int i = 0; i < 8; i += 2) {
        const float2 u = e[i], v = e[i + 1];
        e[i] = make_float2(__fadd_rn(u.x, v.x), __fadd_rn(u.y, v.y));
        e[i + 1] = make_float2(__fsub_rn(u.x, v.x), __fsub_rn(u.y, v.y));
    }
    if constexpr (F) {
        bfly4_one<INV>(&e[0], &e[2], &e[4], &e[6]);
        bfly4<INV, F>(&e[1], &e[3], &e[5], &e[7], __ldg(t + 1), __ldg(t + 3), __ldg(t + 5));
    } else {
#pragma unroll
        for (int j = 0; j < 2; j++)
            bfly4<INV, F>(&e[j], &e[j + 2], &e[j + 4], &e[j + 6], __ldg(t + j), __ldg(t + 2 + j), __ldg(t + 4 + j));
    }
#pragma unroll
    for (int i = 0; i < 8; i++) p[i] = e[i];
}

template <int LOG2N>
struct Line {
    static constexpr int N = 1 << LOG2N;
    static constexpr int LD = N + (N >> 4) + 1;  // padded_len(N)
};

template <bool INV, int LOG2N, int H, bool F>
__device__ __forceinline__ void pass16(float2 *s, int lines, const float2 *tA, const float2 *tB) {
    constexpr int LU = LOG2N - 4, LH = ilog2c(H), LD = Line<LOG2N>::LD;
    const int total = lines << LU;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int line = u >> LU, v = u & ((1 << LU) - 1);
        const int j = v & (H - 1), base = ((v >> LH) << (LH + 4)) + j;
        unit16<INV, H, F>(s + line * LD + padi(base), tA + j, tB + j);
    }
    __syncthreads();
}

template <bool INV, int LOG2N, int H, bool F>
__device__ __forceinline__ void pass4(float2 *s, int lines, const float2 *t) {
    constexpr int LU = LOG2N - 2, LH = ilog2c(H), LD = Line<LOG2N>::LD;
    const int total = lines << LU;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int line = u >> LU, v = u & ((1 << LU) - 1);
        const int j = v & (H - 1), base = ((v >> LH) << (LH + 2)) + j;
        unit4<INV, H, F>(s + line * LD + padi(base), t + j);
    }
    __syncthreads();
}

template <bool INV, int LOG2N, bool F>
__device__ __forceinline__ void pass_head(float2 *s, int lines, const float2 *t) {
    constexpr int LU = LOG2N - 3, LD = Line<LOG2N>::LD;
    const int total = lines << LU;
    for (int u = threadIdx.x; u < total; u += blockDim.x) {
        const int line = u >> LU, v = u & ((1 << LU) - 1);
        unit_head<INV, F>(s + line * LD + padi(v << 3), t);
    }
    __syncthreads();
}

// Stage h's twiddle table starts at h - 1 (even log2) or h - 2 (odd log2,
// after the head's h=2 table) in the concatenated table of
// makeTriTwiddles (radix4.go:45-73).
template <bool INV, int LOG2N, int H, bool F>
__device__ __forceinline__ void passes_from(float2 *s, int lines, const float2 *tri) {
    constexpr int N = 1 << LOG2N;
    constexpr int OFF = (LOG2N & 1) ? H - 2 : H - 1;
    if constexpr (16 * H <= N) {
        pass16<INV, LOG2N, H, F>(s, lines, tri + OFF, tri + OFF + 3 * H);
        passes_from<INV, LOG2N, 16 * H, F>(s, lines, tri);
    } else if constexpr (4 * H <= N) {
        pass4<INV, LOG2N, H, F>(s, lines, tri + OFF);
    }
}

// fftR4Scalar (radix4.go:106-149) over `lines` padded lines of length 2^LOG2N
// in bit-reversed order; ends with a barrier.  F: the fast form's fused
// twiddle products.
template <bool INV, int LOG2N, bool F = false>
__device__ __forceinline__ void line_fft(float2 *s, int lines, const float2 *tri) {
    if constexpr (LOG2N & 1) {
        pass_head<INV, LOG2N, F>(s, lines, tri);
        passes_from<INV, LOG2N, 8, F>(s, lines, tri);
    } else {
        passes_from<INV, LOG2N, 1, F>(s, lines, tri);
    }
}

// The cascade's last pass for log2 n = L: its quarter size and radix (16 or
// 4), following the pass list of line_fft (odd L: the head, then radix-16
// passes from quarter 8; even L: from quarter 1; a trailing radix-4 pass
// when two stages remain).
__host__ __device__ constexpr int last_pass_h(int L) {
    int h = (L & 1) ? 8 : 1, lastH = h;
    while (true) {
        if (16 * h <= (1 << L)) {
            lastH = h;
            h *= 16;
        } else {
            if (4 * h <= (1 << L)) lastH = h;
            return lastH;
        }
    }
}
__host__ __device__ constexpr int last_pass_r(int L) {
    return 16 * last_pass_h(L) <= (1 << L) ? 16 : 4;
}

// Every pass but the last (the fast form scores the last pass's outputs
// from registers); ends with a barrier.
template <bool INV, int LOG2N, int H, bool F>
__device__ __forceinline__ void passes_but_last(float2 *s, int lines, const float2 *tri) {
    constexpr int N = 1 << LOG2N;
    constexpr int OFF = (LOG2N & 1) ? H - 2 : H - 1;
    if constexpr (H != last_pass_h(LOG2N) && 16 * H <= N) {
        pass16<INV, LOG2N, H, F>(s, lines, tri + OFF, tri + OFF + 3 * H);
        passes_but_last<INV, LOG2N, 16 * H, F>(s, lines, tri);
    }
}

template <bool INV, int LOG2N, bool F>
__device__ __forceinline__ void line_fft_but_last(float2 *s, int lines, const float2 *tri) {
    if constexpr (LOG2N & 1) {
        pass_head<INV, LOG2N, F>(s, lines, tri);
        passes_but_last<INV, LOG2N, 8, F>(s, lines, tri);
    } else {
        passes_but_last<INV, LOG2N, 1, F>(s, lines, tri);
    }
}

// The last pass's unit at p (quarter H, R elements at padc(H*i)), computed
// into e without storing.
template <bool INV, int H, int R, bool F>
__device__ __forceinline__ void last_unit(const float2 *p, const float2 *__restrict__ tri, int j, float2 *e) {
#pragma unroll
    for (int i = 0; i < R; i++) e[i] = p[padc(H * i)];
    if constexpr (R == 16) {
        const float2 *tA = tri + j, *tB = tri + 3 * H + j;
        const float2 a1 = __ldg(tA), a2 = __ldg(tA + H), a3 = __ldg(tA + 2 * H);
#pragma unroll
        for (int b = 0; b < 4; b++) bfly4<INV, F>(&e[4 * b], &e[4 * b + 1], &e[4 * b + 2], &e[4 * b + 3], a1, a2, a3);
#pragma unroll
        for (int q = 0; q < 4; q++)
            bfly4<INV, F>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + H * q), __ldg(tB + 4 * H + H * q),
                          __ldg(tB + 8 * H + H * q));
    } else {
        const float2 *t = tri + j;
        bfly4<INV, F>(&e[0], &e[1], &e[2], &e[3], __ldg(t), __ldg(t + H), __ldg(t + 2 * H));
    }
}

// floor(line / cn) for cn in 1..4 and line < 2^15.
__device__ __forceinline__ int div_cn(int line, int cn) {
    const int magic = cn == 1 ? 65536 : (cn == 2 ? 32768 : (cn == 3 ? 21846 : 16384));
    return (line * magic) >> 16;
}

// ------------------------------------------------------------ forward rows

__device__ int g_rows_error = 0;  // a TMA wait that gave up (sticky until read and cleared)

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Stages the CTA's frame rows with the tensor-memory accelerator: thread 0
// arms the mbarrier with the byte count and issues one 2-D box copy (256
// bytes x the map's box rows) per 256 bytes of the rows' span, x rounded
// down to the 16-byte boundary the copy needs (the caller indexes from the
// remainder); every thread then waits, up to ~2^31 cycles (~1 s), after
// which the wait records g_rows_error and returns.
__device__ __noinline__ void tma_stage_rows(const CUtensorMap *map, unsigned char *stage, uint64_t *bar, int xbase,
                                            int y, int nb, int boxRows) {
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                     "r"((unsigned)(nb * 256 * boxRows))
                     : "memory");
        for (int i = 0; i < nb; i++)
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
                    "r"(smem_addr(stage + (size_t)i * 256 * boxRows)),
                "l"(reinterpret_cast<unsigned long long>(map)), "r"(xbase + 256 * i), "r"(y), "r"(smem_addr(bar))
                : "memory");
    }
    __syncthreads();
    const uint32_t a = smem_addr(bar);
    const long long t0 = clock64();
    for (unsigned it = 0;; it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
            "selp.b32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(a)
            : "memory");
        if (ok) break;
        if ((it & 255u) == 255u && clock64() - t0 > (1ll << 31)) {
            atomicExch(&g_rows_error, 1);
            break;
        }
    }
}

template <int LOG2N, bool F>
__global__ void __launch_bounds__(256) k_fwd_rows_t(FwdRowsArgs a, const __grid_constant__ CUtensorMap map) {
    griddep_wait();
    griddep_launch();
    constexpr int N = 1 << LOG2N, LD = Line<LOG2N>::LD, HALF = N / 2;
    extern __shared__ float2 smem[];
    const FftClass &fc = a.fc;
    const int tile = fc.tileFirst + blockIdx.y;
    const TileBox b = tile_box(a.g, tile);
    const int nrows = min(b.loadH, fc.dftH);
    const int pair0 = blockIdx.x * a.pairsPerCta;
    if (2 * pair0 >= nrows) return;
    const int cnEff = a.cnDev ? min(*a.cnDev, a.chanCount) : a.chanCount;
    const int cn = min(cnEff - a.chanFirst, a.chanGroup);  // channels of this launch's group
    if (cn <= 0) return;
    const int P = min(a.pairsPerCta, (nrows - 2 * pair0 + 1) >> 1);
    const int lines = P * cn;
    const int tid = threadIdx.x, nt = blockDim.x;
    const long long istride = a.istride;
    const uint8_t *img0 = a.img + (long long)(b.y0 + 2 * pair0) * istride + (long long)b.x0 * a.step;
    float subv[4];
    if (a.selfSums) {
        // the template's own channel sums (this launch's one tile is the
        // whole template): exact integers, reduced per warp then per CTA
        __shared__ unsigned long long ssum[4];
        if (tid < 4) ssum[tid] = 0ull;
        __syncthreads();
        unsigned long long sv[4] = {0ull, 0ull, 0ull, 0ull};
        const uint8_t *t0 = a.img + (long long)b.y0 * istride + (long long)b.x0 * a.step;
        const int npx = b.loadW * b.loadH;
        for (int i = tid; i < npx; i += nt) {
            const int y = i / b.loadW, x = i - y * b.loadW;
            const uint8_t *q = t0 + (long long)y * istride + (long long)x * a.step;
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (c < a.step) sv[c] += q[c];
        }
#pragma unroll
        for (int c = 0; c < 4; c++) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sv[c] += __shfl_down_sync(0xffffffffu, sv[c], o);
            if ((tid & 31) == 0 && sv[c]) atomicAdd(&ssum[c], sv[c]);
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 4; c++) subv[c] = __fdiv_rn(__ull2float_rn(ssum[c]), a.subDiv);
    } else {
#pragma unroll
        for (int g = 0; g < 4; g++)
            subv[g] = a.subSums ? __fdiv_rn(__ull2float_rn(a.subSums[g]), a.subDiv) : a.sub[g];
    }
    // TMA: the CTA's rows land in shared memory first (box i holds bytes
    // [xbase + 256 i, +256) of each of the box's rows)
    __shared__ __align__(8) uint64_t tmaBar;
    const int boxRows = 2 * a.pairsPerCta;
    // (128-byte aligned whatever the dynamic shared memory's base)
    const unsigned char *stage = reinterpret_cast<const unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem) + a.tmaSmemOff + 127) & ~uintptr_t(127));
    int tmaOff = 0;
    if (a.tma) {
        const int xbyte = b.x0 * a.step, xbase = xbyte & ~15;
        tmaOff = xbyte - xbase;
        const int nb = (tmaOff + b.loadW * a.step + 255) >> 8;
        tma_stage_rows(&map, const_cast<unsigned char *>(stage), &tmaBar, xbase, b.y0 + 2 * pair0, nb, boxRows);
    }
    // Pack rows r (real part) and r+1 (imaginary part) of every channel of
    // the group, each pixel read once for all of them.
    for (int it = tid; it < (P << LOG2N); it += nt) {
        const int p = it >> LOG2N, x = it & (N - 1);
        float va[4] = {0.f, 0.f, 0.f, 0.f}, vb[4] = {0.f, 0.f, 0.f, 0.f};
        if (x < b.loadW) {
            const bool two = 2 * (pair0 + p) + 1 < b.loadH;
            const uint8_t *q = img0 + (long long)(2 * p) * istride + (long long)x * a.step;
            long long qstride = istride;
            if (a.tma) {
                const int o = tmaOff + x * a.step;
                q = stage + (size_t)(o >> 8) * 256 * boxRows + (size_t)(2 * p) * 256 + (o & 255);
                qstride = 256;
            }
            if (a.pix32) {
                const unsigned int w0 = *reinterpret_cast<const unsigned int *>(q);
                const unsigned int w1 = two ? *reinterpret_cast<const unsigned int *>(q + qstride) : 0u;
#pragma unroll
                for (int g = 0; g < 4; g++) {
                    const int sh = 8 * (a.chanFirst + g);
                    va[g] = (float)((w0 >> (sh & 31)) & 255u);
                    vb[g] = (float)((w1 >> (sh & 31)) & 255u);
                }
            } else {
#pragma unroll
                for (int g = 0; g < 4; g++)
                    if (g < cn) {
                        va[g] = (float)q[a.chanFirst + g];
                        if (two) vb[g] = (float)q[qstride + a.chanFirst + g];
                    }
            }
            // pixel * mul - sub: exact for the integer operands used (x1 - 0
            // leaves the reference's samples untouched); the missing second
            // row of an odd tail stays zero
#pragma unroll
            for (int g = 0; g < 4; g++) {
                const float sg = subv[(a.chanFirst + g) & 3];
                va[g] = __fsub_rn(__fmul_rn(va[g], a.mul), sg);
                vb[g] = two ? __fsub_rn(__fmul_rn(vb[g], a.mul), sg) : 0.f;
            }
        }
        float2 *d = smem + (p * cn) * LD + padi(brevn<LOG2N>(x));
#pragma unroll
        for (int g = 0; g < 4; g++)
            if (g < cn) d[g * LD] = make_float2(va[g], vb[g]);
    }
    __syncthreads();
    // Untangle (impl.go:331-341) into the two real-row spectra at their
    // bit-reversed column-transform slots.
    const int hwp = fc.hwp, log2H = fc.log2H;
    const size_t chanStride = (size_t)fc.dftH * hwp;
    float2 *tbase = a.spec + (size_t)(tile - fc.tileFirst) * a.cnS * chanStride;
    auto rows = [&](int line, float2 *&ra, float2 *&rb) {
        const int p = div_cn(line, cn), k = a.chanFirst + line - p * cn;
        const int r = 2 * (pair0 + p);
        float2 *cb = tbase + (size_t)k * chanStride;
        ra = cb + (size_t)brev_bits(r, log2H) * hwp;
        rb = cb + (size_t)brev_bits(r + 1, log2H) * hwp;
    };
    // spectrum column kk of both rows from z[kk] and its mirror n = z[(N - kk) mod N]
    auto emit = [&](float2 *ra, float2 *rb, int kk, float2 z, float2 n) {
        ra[kk] = make_float2(__fmul_rn(0.5f, __fadd_rn(z.x, n.x)), __fmul_rn(0.5f, __fsub_rn(z.y, n.y)));
        rb[kk] = make_float2(__fmul_rn(0.5f, __fadd_rn(z.y, n.y)), __fmul_rn(0.5f, __fsub_rn(n.x, z.x)));
    };
    if constexpr (last_pass_r(LOG2N) == 4) {
        // A radix-4 last pass (quarter H = N/4) fused with the untangle: unit
        // j holds z[j + H*i], and the mirror of each of its outputs below N/2
        // lies in unit H - j, so one item runs units j and H - j and writes
        // their four columns of both rows from registers (j = 0 and j = H/2
        // are their own mirrors; unit 0 also holds z[N/2]).  The same rounded
        // operations as the separate pass and untangle.
        line_fft_but_last<false, LOG2N, F>(smem, lines, fc.triW);
        constexpr int H = last_pass_h(LOG2N), OFF = (LOG2N & 1) ? H - 2 : H - 1, PER = H / 2 + 1;
        const float2 *tri = fc.triW + OFF;
        for (int it = tid; it < lines * PER; it += nt) {
            const int line = it / PER, j = it - line * PER;
            float2 *ra, *rb;
            rows(line, ra, rb);
            const float2 *zl = smem + line * LD;
            float2 za[4];
            last_unit<false, H, 4, F>(zl + padi(j), tri, j, za);
            if (j == 0) {
                emit(ra, rb, 0, za[0], za[0]);
                emit(ra, rb, H, za[1], za[3]);
                const float2 zk = za[2];  // kk = N/2
                ra[HALF] = make_float2(__fmul_rn(0.5f, __fadd_rn(zk.x, zk.x)), __fmul_rn(0.5f, __fsub_rn(zk.y, zk.y)));
                rb[HALF] = make_float2(__fmul_rn(0.5f, __fadd_rn(zk.y, zk.y)), __fmul_rn(0.5f, __fsub_rn(zk.x, zk.x)));
            } else if (j == H / 2) {
                emit(ra, rb, j, za[0], za[3]);
                emit(ra, rb, j + H, za[1], za[2]);
            } else {
                const int jp = H - j;
                float2 zb[4];
                last_unit<false, H, 4, F>(zl + padi(jp), tri, jp, zb);
                emit(ra, rb, j, za[0], zb[3]);
                emit(ra, rb, j + H, za[1], zb[2]);
                emit(ra, rb, jp, zb[0], za[3]);
                emit(ra, rb, jp + H, zb[1], za[2]);
            }
        }
        return;
    }
    line_fft<false, LOG2N, F>(smem, lines, fc.triW);
    // two spectrum columns kk, kk+1 per item: one 16-byte store per row
    for (int it = tid; it < (lines << (LOG2N - 2)); it += nt) {
        const int line = it >> (LOG2N - 2), kk = 2 * (it & (HALF / 2 - 1));
        float2 *ra, *rb;
        rows(line, ra, rb);
        const float2 *zl = smem + line * LD;
        const float2 z0 = zl[padi(kk)], n0 = zl[padi((N - kk) & (N - 1))];
        const float2 z1 = zl[padi(kk + 1)], n1 = zl[padi(N - kk - 1)];
        *reinterpret_cast<float4 *>(ra + kk) =
            make_float4(__fmul_rn(0.5f, __fadd_rn(z0.x, n0.x)), __fmul_rn(0.5f, __fsub_rn(z0.y, n0.y)),
                        __fmul_rn(0.5f, __fadd_rn(z1.x, n1.x)), __fmul_rn(0.5f, __fsub_rn(z1.y, n1.y)));
        *reinterpret_cast<float4 *>(rb + kk) =
            make_float4(__fmul_rn(0.5f, __fadd_rn(z0.y, n0.y)), __fmul_rn(0.5f, __fsub_rn(n0.x, z0.x)),
                        __fmul_rn(0.5f, __fadd_rn(z1.y, n1.y)), __fmul_rn(0.5f, __fsub_rn(n1.x, z1.x)));
    }
    for (int line = tid; line < lines; line += nt) {  // kk = N/2
        float2 *ra, *rb;
        rows(line, ra, rb);
        const float2 zk = smem[line * LD + padi(HALF)];
        ra[HALF] = make_float2(__fmul_rn(0.5f, __fadd_rn(zk.x, zk.x)), __fmul_rn(0.5f, __fsub_rn(zk.y, zk.y)));
        rb[HALF] = make_float2(__fmul_rn(0.5f, __fadd_rn(zk.y, zk.y)), __fmul_rn(0.5f, __fsub_rn(zk.x, zk.x)));
    }
}

// ------------------------------------------------------------ inverse rows

// The generic inverse-rows kernel (cvm_kernels.cu) with the length fixed:
// combine (impl.go:405-413) reads each spectrum pair once and writes both
// z[kk] and its mirror z[N-kk]; the channels accumulate in channel order;
// the epilogue scores with the per-result (t, den) lanes and keeps
// first-occurrence extrema merged by each member's last CTA.
template <int LOG2N, bool FAST>
// Occupancy: the fast form's radix-16 last pass budgets two CTAs per SM;
// its radix-4 last pass four (64 registers, with four row pairs per CTA in
// fleets: rows_fast_pairs), the exact form three.
__global__ void __launch_bounds__(256, FAST ? (last_pass_r(LOG2N) == 16 ? 2 : 4) : 3) k_inv_rows_t(InvArgs a) {
    griddep_wait();
    constexpr int N = 1 << LOG2N, LD = Line<LOG2N>::LD, HALF = N / 2;
    constexpr int XIT = (N + kThreads - 1) / kThreads;  // result columns per thread
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
    const int hwp = fc.hwp, log2H = fc.log2H;
    const int tid = threadIdx.x;
    const bool flat = Pm.flat != 0;
    const float denFlat = near_flat_den(m.tw, m.th, Pm.templNorm);  // fast form: near-flat windows below it
    float *acc = reinterpret_cast<float *>(smem + (size_t)a.pairsPerCta * LD);  // [P][2][N]
    Ext e;
    ext_init(e);
    // the fast form's scratch holds one channel-summed correlation per tile
    constexpr bool fast = FAST;
    // a radix-4 last pass is fused with the scoring (both forms; not for
    // the fixed-scratch entry point, which takes the raw correlation)
    // (a radix-16 last pass only in the fast form, which budgets the
    // registers for it: two CTAs per SM)
    const bool fuse = (last_pass_r(LOG2N) == 4 || FAST) && a.ms.lanes != nullptr;
    if (P > 0 && !flat) {
        const int cn = fast ? 1 : Pm.cn;
        const size_t chanStride = (size_t)fc.dftH * hwp;
        const float2 *scr = a.ms.scratch[a.cls] + (size_t)slot * a.ms.scratchStride[a.cls];
        for (int k = 0; k < cn; k++) {
            const float2 *cb = scr + ((size_t)tileLocal * a.cnS + k) * chanStride;
            // two spectrum columns kk, kk+1 per item (16-byte loads)
            const int total = P << (LOG2N - 2);
#pragma unroll 4
            for (int it = tid; it < total; it += kThreads) {
                const int p = it >> (LOG2N - 2), kk = 2 * (it & (HALF / 2 - 1));
                const int r = 2 * (pair0 + p);
                const float4 u = __ldg(reinterpret_cast<const float4 *>(cb + (size_t)brev_bits(r, log2H) * hwp + kk));
                const float4 v =
                    __ldg(reinterpret_cast<const float4 *>(cb + (size_t)brev_bits(r + 1, log2H) * hwp + kk));
                float2 *zl = smem + p * LD;
                zl[padi(brevn<LOG2N>(kk))] = make_float2(__fsub_rn(u.x, v.y), __fadd_rn(u.y, v.x));
                zl[padi(brevn<LOG2N>(kk + 1))] = make_float2(__fsub_rn(u.z, v.w), __fadd_rn(u.w, v.z));
                if (kk > 0)
                    zl[padi(brevn<LOG2N>(N - kk))] = make_float2(__fadd_rn(u.x, v.y), __fsub_rn(v.x, u.y));
                zl[padi(brevn<LOG2N>(N - kk - 1))] = make_float2(__fadd_rn(u.z, v.w), __fsub_rn(v.z, u.w));
            }
            if (tid < P) {
                const int r = 2 * (pair0 + tid);
                const float2 u = __ldg(cb + (size_t)brev_bits(r, log2H) * hwp + HALF);
                const float2 v = __ldg(cb + (size_t)brev_bits(r + 1, log2H) * hwp + HALF);
                smem[tid * LD + padi(brevn<LOG2N>(HALF))] = make_float2(__fsub_rn(u.x, v.y), __fadd_rn(u.y, v.x));
            }
            __syncthreads();
            if (fuse && k == cn - 1) {
                // the last channel's last pass runs in the epilogue, which
                // finishes the channel sum and scores from registers
                line_fft_but_last<true, LOG2N, FAST>(smem, P, fc.triW);
                break;
            }
            line_fft<true, LOG2N, FAST>(smem, P, fc.triW);
            if (fast) break;  // one channel: the epilogue reads the transformed lines directly
            for (int p = 0; p < P; p++) {
                const float2 *zl = smem + p * LD;
                float *a0 = acc + (size_t)(2 * p) * N, *a1 = a0 + N;
#pragma unroll
                for (int q = 0; q < XIT; q++) {
                    const int x = tid + q * kThreads;
                    if (x < bw) {
                        const float2 z = zl[padi(x)];
                        if (k == 0) {
                            a0[x] = z.x;
                            a1[x] = z.y;
                        } else {
                            a0[x] = __fadd_rn(a0[x], z.x);
                            a1[x] = __fadd_rn(a1[x], z.y);
                        }
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
#pragma unroll
                for (int q = 0; q < XIT; q++) {
                    const int x = tid + q * kThreads;
                    if (x < bw) corr[(size_t)(tb.y0 + 2 * pair0 + rr) * m.rw + tb.x0 + x] = acc[(size_t)rr * N + x];
                }
        }
        return;
    }
    if (FAST && fuse && P > 0 && !flat && !a.ms.map && !a.ms.anyRoi) {
        // The fast form without a score map or regions of interest (every
        // fleet FindAll): the same units, scores and visiting order as the
        // general epilogue below, with the CTA-local raster index of a result
        // (row within the CTA x N + x, ascending as the general epilogue's
        // global index does) kept in 32 bits and widened once at the end.
        constexpr int LH = last_pass_h(LOG2N), LR = last_pass_r(LOG2N);
        constexpr int LLR = LR == 16 ? 4 : 2, LLH = ilog2c(LH), LU = LOG2N - LLR;
        constexpr int OFF = (LOG2N & 1) ? LH - 2 : LH - 1;
        const float *dens = reinterpret_cast<const float *>(a.ms.lanes + (size_t)slot * a.ms.lanesStride);
        // a fleet wave with the frame's summed-area table forms each
        // window's den here (no statistics kernel ran for it)
        const bool ownStats = a.ms.sat != nullptr;
        float minV = FLT_MAX, maxV = -FLT_MAX;
        int minL = INT_MAX, maxL = INT_MAX;
        for (int u = tid; u < (P << LU); u += kThreads) {
            const int line = u >> LU, v = u & ((1 << LU) - 1);
            const int j = v & (LH - 1), base = ((v >> LLH) << (LLH + LLR)) + j;
            const int rl = 2 * line;                          // CTA-local row of the real part
            const bool odd = 2 * (pair0 + line) + 1 < bh;     // the imaginary part's row exists
            const int y0 = tb.y0 + 2 * (pair0 + line);
            const float *d0 = dens + (long long)y0 * m.rw + tb.x0;
            float den0[LR], den1[LR];
            if (ownStats) {
#pragma unroll
                for (int i = 0; i < LR; i++) {
                    const int x = base + LH * i;
                    den0[i] = x < bw ? sat_den(a.ms, m, Pm, y0, tb.x0 + x) : 0.f;
                    den1[i] = (x < bw && odd) ? sat_den(a.ms, m, Pm, y0 + 1, tb.x0 + x) : 0.f;
                }
            } else {
#pragma unroll
                for (int i = 0; i < LR; i++) {
                    const int x = base + LH * i;
                    den0[i] = x < bw ? __ldg(d0 + x) : 0.f;
                    den1[i] = (x < bw && odd) ? __ldg(d0 + m.rw + x) : 0.f;
                }
            }
            float2 z[LR];
            last_unit<true, LH, LR, FAST>(smem + line * LD + padi(base), fc.triW + OFF, j, z);
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (h == 1 && !odd) break;
                const int l0 = (rl + h) * N;
#pragma unroll
                for (int i = 0; i < LR; i++) {
                    const int x = base + LH * i;
                    if (x < bw) {
                        const float sc = score_fast(h ? z[i].y : z[i].x, h ? den1[i] : den0[i], denFlat);
                        if (sc < minV) {
                            minV = sc;
                            minL = l0 + x;
                        }
                        if (sc > maxV) {
                            maxV = sc;
                            maxL = l0 + x;
                        }
                    }
                }
            }
        }
        // widen: CTA-local (row, x) -> the member's raster index
        auto widen = [&](int l) {
            return l == INT_MAX ? LLONG_MAX
                                : (long long)(tb.y0 + 2 * pair0 + (l >> LOG2N)) * m.rw + tb.x0 + (l & (N - 1));
        };
        e.minV = minV;
        e.maxV = maxV;
        e.minI = widen(minL);
        e.maxI = widen(maxL);
    } else if (fuse && P > 0 && !flat) {
        // The last pass of every line, each unit's outputs scored straight
        // from registers: x = base + H*i of line p are results x of rows 2p
        // (real part) and 2p+1 (imaginary part).  A thread owns at most one
        // unit per line and visits lines in order, so its results ascend in
        // raster order (ext_add_inc).  The exact form adds the earlier
        // channels' sum to the last channel's output (the accumulation's
        // own rounded add, in channel order) and subtracts t, as the
        // unfused epilogue does.
        constexpr int LH = last_pass_h(LOG2N), LR = last_pass_r(LOG2N);
        constexpr int LLR = LR == 16 ? 4 : 2, LLH = ilog2c(LH), LU = LOG2N - LLR;
        constexpr int OFF = (LOG2N & 1) ? LH - 2 : LH - 1;
        const float2 *lanes = a.ms.lanes + (size_t)slot * a.ms.lanesStride;
        const float *dens = reinterpret_cast<const float *>(lanes);
        const int cnSum = FAST ? 1 : Pm.cn;
        float *map = a.ms.map;
        const int xlo = m.roiX0 - tb.x0, xhi = m.roiX1 - tb.x0;
        for (int u = tid; u < (P << LU); u += kThreads) {
            const int line = u >> LU, v = u & ((1 << LU) - 1);
            const int j = v & (LH - 1), base = ((v >> LLH) << (LLH + LLR)) + j;
            // the unit's (t, den) values first: their loads overlap its butterflies
            long long rowBase[2];
            float2 dv[2][LR];
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const int yy = tb.y0 + 2 * (pair0 + line) + half;
                rowBase[half] = (long long)yy * m.rw + tb.x0;
#pragma unroll
                for (int i = 0; i < LR; i++) {
                    const int x = base + LH * i;
                    const bool in = x < bw && 2 * (pair0 + line) + half < bh;
                    if (FAST)
                        dv[half][i] = make_float2(0.f, in ? __ldg(dens + rowBase[half] + x) : 0.f);
                    else
                        dv[half][i] = in ? __ldg(lanes + rowBase[half] + x) : make_float2(0.f, 0.f);
                }
            }
            float2 z[LR];
            last_unit<true, LH, LR, FAST>(smem + line * LD + padi(base), fc.triW + OFF, j, z);
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const int r = 2 * (pair0 + line) + half;
                if (r >= bh) break;
                const int yy = tb.y0 + r;
                if (yy < m.roiY0 || yy >= m.roiY1) continue;
#pragma unroll
                for (int i = 0; i < LR; i++) {
                    const int x = base + LH * i;
                    if (x < bw) {
                        float num = half ? z[i].y : z[i].x;
                        if (!FAST) {
                            if (cnSum > 1) num = __fadd_rn(acc[(size_t)(2 * line + half) * N + x], num);
                            num = __fsub_rn(num, dv[half][i].x);
                        }
                        const float den = dv[half][i].y;
                        const float score = FAST ? score_fast(num, den, denFlat) : score_exact(num, den);
                        if (map) map[rowBase[half] + x] = score;
                        if (x >= xlo && x < xhi) ext_add_inc(e, score, rowBase[half] + x);
                    }
                }
            }
        }
    } else if (P > 0) {
        const float2 *lanes = a.ms.lanes + (size_t)slot * a.ms.lanesStride;
        float *map = a.ms.map;
        const int xlo = m.roiX0 - tb.x0, xhi = m.roiX1 - tb.x0;
        for (int rr = 0; rr < 2 * P; rr++) {
            const int r = 2 * pair0 + rr;
            if (r >= bh) break;
            const long long rowBase = (long long)(tb.y0 + r) * m.rw + tb.x0;
            if (tb.y0 + r < m.roiY0 || tb.y0 + r >= m.roiY1) continue;  // no map here (only fleets have ROIs)
            // (t, den); the fast form stores den alone, one float per result
            float2 td[XIT];
#pragma unroll
            for (int q = 0; q < XIT; q++) {
                const int x = tid + q * kThreads;
                if (fast)
                    td[q] = make_float2(0.f, (!flat && x < bw) ? __ldg(reinterpret_cast<const float *>(lanes) + rowBase + x)
                                                               : 0.f);
                else
                    td[q] = (!flat && x < bw) ? __ldg(lanes + rowBase + x) : make_float2(0.f, 0.f);
            }
            const float2 *zl = smem + (rr >> 1) * LD;  // fast form: row rr is line rr/2's real or imaginary part
#pragma unroll
            for (int q = 0; q < XIT; q++) {
                const int x = tid + q * kThreads;
                if (x < bw) {
                    float score = 1.f;
                    if (!flat) {
                        float num;
                        if (fast) {
                            const float2 z = zl[padi(x)];
                            num = (rr & 1) ? z.y : z.x;
                        } else {
                            num = __fsub_rn(acc[(size_t)rr * N + x], td[q].x);
                        }
                        const float den = td[q].y;
                        score = fast ? score_fast(num, den, denFlat) : score_exact(num, den);
                    }
                    if (map) map[rowBase + x] = score;
                    // rows ascend, and x ascends within a row: increasing indices
                    if (x >= xlo && x < xhi) ext_add_inc(e, score, rowBase + x);
                }
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
    for (int i = tid; i < a.nparts; i += kThreads) {
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

template <int L>
void fwd_one(const FwdRowsArgs &a, const CUtensorMap &map, dim3 grid, int threads, size_t smem, cudaStream_t st) {
    if (a.fma) {
        set_smem(k_fwd_rows_t<L, true>, smem);
        launch_k(k_fwd_rows_t<L, true>, grid, dim3(threads), smem, st, a, map);
    } else {
        set_smem(k_fwd_rows_t<L, false>, smem);
        launch_k(k_fwd_rows_t<L, false>, grid, dim3(threads), smem, st, a, map);
    }
}

template <int L>
void inv_one(const InvArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    if (a.ms.form) {
        set_smem(k_inv_rows_t<L, true>, smem);
        launch_k(k_inv_rows_t<L, true>, grid, dim3(kThreads), smem, st, a);
    } else {
        set_smem(k_inv_rows_t<L, false>, smem);
        launch_k(k_inv_rows_t<L, false>, grid, dim3(kThreads), smem, st, a);
    }
}

}  // namespace

bool rows_fixed_length(int log2n) { return log2n >= 5 && log2n <= 12; }

// Elements per CTA of a fleet wave's fast-form inverse rows: a radix-4
// last pass runs four CTAs per SM, whose shared memory holds 4096 elements
// each (C4's 78-member waves of 1024-point rows: 3.56 -> 3.38 ms per frame
// against 8192 at three CTAs); a radix-16 last pass keeps 8192 at two.
int rows_fast_wave_elems(int log2n) { return log2n >= 5 && log2n <= 12 && last_pass_r(log2n) == 4 ? 4096 : 8192; }

void launch_fwd_rows_fixed(const FwdRowsArgs &a, const CUtensorMap &map, dim3 grid, int threads, size_t smem,
                           cudaStream_t st) {
    switch (a.fc.log2n) {
        case 5: fwd_one<5>(a, map, grid, threads, smem, st); break;
        case 6: fwd_one<6>(a, map, grid, threads, smem, st); break;
        case 7: fwd_one<7>(a, map, grid, threads, smem, st); break;
        case 8: fwd_one<8>(a, map, grid, threads, smem, st); break;
        case 9: fwd_one<9>(a, map, grid, threads, smem, st); break;
        case 10: fwd_one<10>(a, map, grid, threads, smem, st); break;
        case 11: fwd_one<11>(a, map, grid, threads, smem, st); break;
        default: fwd_one<12>(a, map, grid, threads, smem, st); break;
    }
}

bool encode_frame_map(CUtensorMap *map, const void *img, long long istride, long long wBytes, int h, int boxRows) {
    static PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
    static int tried = 0;
    if (!tried) {
        tried = 1;
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            enc = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        else
            cudaGetLastError();
    }
    if (!enc || boxRows < 1 || boxRows > 256) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)wBytes, (cuuint64_t)h};
    const cuuint64_t strides[1] = {(cuuint64_t)istride};
    const cuuint32_t box[2] = {256u, (cuuint32_t)boxRows};
    const cuuint32_t estr[2] = {1u, 1u};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, const_cast<void *>(img), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

int rows_error_read_clear() {
    int v = 0, z = 0;
    if (cudaMemcpyFromSymbol(&v, g_rows_error, sizeof v) != cudaSuccess) return -1;
    if (v) cudaMemcpyToSymbol(g_rows_error, &z, sizeof z);
    return v;
}

void launch_inv_rows_fixed(const InvArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    switch (a.fc.log2n) {
        case 5: inv_one<5>(a, grid, smem, st); break;
        case 6: inv_one<6>(a, grid, smem, st); break;
        case 7: inv_one<7>(a, grid, smem, st); break;
        case 8: inv_one<8>(a, grid, smem, st); break;
        case 9: inv_one<9>(a, grid, smem, st); break;
        case 10: inv_one<10>(a, grid, smem, st); break;
        case 11: inv_one<11>(a, grid, smem, st); break;
        default: inv_one<12>(a, grid, smem, st); break;
    }
}

}  // namespace cvm
