// cvm_cols.cu -- the column transforms specialised on the transform height.
//
// colsR4Go (radix4cols.go:35-125) forward, mulConjGo (impl.go:376-388) and
// colsR4Go inverse for dftH = 2^5 .. 2^12 over strips of SC columns, one
// kernel instance per (mode, height).  The arithmetic is the generic
// kernels' (cvm_kernels.cu): the same butterflies, twiddles and rounded op
// order.  With the height fixed, every pass's radix, quarter size and
// twiddle offset are compile-time constants, so each unit addresses its
// elements at constant offsets -- also through the inverse's bit-reversed
// row map, because a unit's base and its element offsets occupy disjoint
// bits (brev(base + h*i) = brev(base) + brev(h*i)).
//
// Storage relabelling (radix4cols.go:12-24): the forward cascade reads the
// forward-rows output in slot order (slot s holds logical row brev(s)) and
// leaves frequency rows in natural order; the inverse cascade reads
// logical element i from row brev(i) and leaves spatial row y at logical
// y, stored to slot brev(y) of the scratch spectrum.
//
// Middle sweep.  The forward cascade's last pass and the inverse cascade's
// first pass act on the same rows: with M = 16 (or 8) and S = dftH / M,
// the rows {B + S*c : c < M} (B < S) hold complete butterflies of the
// forward's last pass, and through the bit reversal they are one
// contiguous block of logical slots of the inverse's first pass.  So one
// sweep runs both passes and the conj-multiply in registers:
//   even log2, last pass radix 16 (quarter S)   M = 16, inverse radix-16 unit
//   even log2, last pass radix 4 (quarter 4S)   M = 16, four radix-4 units
//   odd log2, last pass radix 4 (quarter 2S)    M = 8,  two radix-4 units, inverse head
//   odd log2, last pass radix 16 (quarter S)    M = 16, two inverse heads (even / odd c)
// where the inverse "head" is the radix-2 stage plus the h=2 radix-4 stage
// on 8 contiguous logical slots.
#include <type_traits>

#include "cvm_device.cuh"

namespace cvm {
namespace {

enum { KHEAD = 0, K16 = 1, K4 = 2 };

__host__ __device__ constexpr int ilog2k(int v) { return v <= 1 ? 0 : 1 + ilog2k(v >> 1); }

__host__ __device__ constexpr int brevk(int x, int bits) {
    int r = 0;
    for (int i = 0; i < bits; i++) r |= ((x >> i) & 1) << (bits - 1 - i);
    return r;
}

// The cascade's pass list for log2 height L (fftR4Scalar, radix4.go:106-149):
// odd L: the head, then radix-16 passes from quarter 8; even L: radix-16
// passes from quarter 1; a trailing radix-4 pass when two stages remain.
__host__ __device__ constexpr int npass(int L) {
    int n = 0, h = 1;
    if (L & 1) {
        n = 1;
        h = 8;
    }
    while (16 * h <= (1 << L)) {
        n++;
        h *= 16;
    }
    if (4 * h <= (1 << L)) n++;
    return n;
}

// quarter size of pass p (1 for the head)
__host__ __device__ constexpr int pass_h(int L, int p) {
    int h = 1, i = 0;
    if (L & 1) {
        if (p == 0) return 1;
        i = 1;
        h = 8;
    }
    while (16 * h <= (1 << L)) {
        if (i == p) return h;
        i++;
        h *= 16;
    }
    return h;
}

__host__ __device__ constexpr int pass_kind(int L, int p) {
    return ((L & 1) && p == 0) ? KHEAD : (16 * pass_h(L, p) <= (1 << L) ? K16 : K4);
}

// Stage h's table starts at h - 1 (even L) or h - 2 (odd L, after the
// head's h=2 table) in makeTriTwiddles' concatenation (radix4.go:45-73).
__host__ __device__ constexpr int tw_off(int L, int h) { return (L & 1) ? h - 2 : h - 1; }

template <bool INV, int H, bool F = false>
__device__ __forceinline__ void math16(float2 *e, const float2 *__restrict__ t) {
    const float2 *tB = t + 3 * H;
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
        return;
    }
    const float2 a1 = __ldg(t), a2 = __ldg(t + H), a3 = __ldg(t + 2 * H);
#pragma unroll
    for (int b = 0; b < 4; b++) bfly4<INV, F>(&e[4 * b], &e[4 * b + 1], &e[4 * b + 2], &e[4 * b + 3], a1, a2, a3);
#pragma unroll
    for (int q = 0; q < 4; q++)
        bfly4<INV, F>(&e[q], &e[q + 4], &e[q + 8], &e[q + 12], __ldg(tB + H * q), __ldg(tB + 4 * H + H * q),
                   __ldg(tB + 8 * H + H * q));
}

template <bool INV, int H, bool F = false>
__device__ __forceinline__ void math4(float2 *e, const float2 *__restrict__ t) {
    bfly4<INV, F>(&e[0], &e[1], &e[2], &e[3], __ldg(t), __ldg(t + H), __ldg(t + 2 * H));
}

template <bool INV, bool F = false>
__device__ __forceinline__ void math_head(float2 *e, const float2 *__restrict__ t) {
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
}

__device__ __forceinline__ float2 mul_conj(float2 av, float2 bv) {
    return make_float2(__fadd_rn(__fmul_rn(av.x, bv.x), __fmul_rn(av.y, bv.y)),
                       __fsub_rn(__fmul_rn(av.y, bv.x), __fmul_rn(av.x, bv.y)));
}

// ---------------------------------------------------------------- element I/O
// A unit's R elements are rows base + STEP*i (i < R) of its column c.

template <int LSC>
struct SmemNat {  // row r at s[(r << LSC) + c]
    float2 *s;
    template <int R, int STEP>
    __device__ __forceinline__ void load(float2 *e, int c, int base) const {
        const float2 *p = s + (base << LSC) + c;
#pragma unroll
        for (int i = 0; i < R; i++) e[i] = p[(STEP * i) << LSC];
    }
    template <int R, int STEP>
    __device__ __forceinline__ void store(const float2 *e, int c, int base) const {
        float2 *p = s + (base << LSC) + c;
#pragma unroll
        for (int i = 0; i < R; i++) p[(STEP * i) << LSC] = e[i];
    }
};

template <int L, int LSC>
struct SmemRev {  // logical element i at row brev(i)
    float2 *s;
    template <int R, int STEP>
    __device__ __forceinline__ void load(float2 *e, int c, int base) const {
        const float2 *p = s + (brev_bits(base, L) << LSC) + c;
#pragma unroll
        for (int i = 0; i < R; i++) e[i] = p[brevk(STEP * i, L) << LSC];
    }
    template <int R, int STEP>
    __device__ __forceinline__ void store(const float2 *e, int c, int base) const {
        float2 *p = s + (brev_bits(base, L) << LSC) + c;
#pragma unroll
        for (int i = 0; i < R; i++) p[brevk(STEP * i, L) << LSC] = e[i];
    }
};

// Forward-rows output: slot s (logical row brev(s)); rows never loaded
// are zero (impl.go:352-356).
template <int L>
struct GlobalSlots {
    const float2 *src;
    int hwp, wv, loaded;
    template <int R, int STEP>
    __device__ __forceinline__ void load(float2 *e, int c, int base) const {
        const int rb = brev_bits(base, L);
        const float2 *p = src + (size_t)base * hwp + c;
#pragma unroll
        for (int i = 0; i < R; i++)
            e[i] = (c < wv && rb + brevk(STEP * i, L) < loaded) ? p[(size_t)(STEP * i) * hwp]
                                                                : make_float2(0.f, 0.f);
    }
};

// Natural-order spectrum out (mode 0), optionally scaled.
struct GlobalNat {
    float2 *dst;
    int hwp, wv;
    float sc;
    template <int R, int STEP>
    __device__ __forceinline__ void store(const float2 *e, int c, int base) const {
        if (c >= wv) return;
        float2 *p = dst + (size_t)base * hwp + c;
#pragma unroll
        for (int i = 0; i < R; i++) {
            float2 v = e[i];
            if (sc != 1.0f) v = make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
            p[(size_t)(STEP * i) * hwp] = v;
        }
    }
};

// Inverse output: logical element i (spatial row i) to slot brev(i), rows
// below rowsOut only.
template <int L>
struct GlobalInv {
    float2 *dst;
    int hwp, wv, rowsOut;
    template <int R, int STEP>
    __device__ __forceinline__ void store(const float2 *e, int c, int base) const {
        if (c >= wv) return;
        const int rb = brev_bits(base, L);
#pragma unroll
        for (int i = 0; i < R; i++)
            if (base + STEP * i < rowsOut) dst[(size_t)(rb + brevk(STEP * i, L)) * hwp + c] = e[i];
    }
};

// One cascade pass p over all columns of the strip.  Ends with a barrier.
template <bool INV, int L, int P, int LSC, bool F, typename LDF, typename STF>
__device__ __forceinline__ void col_pass(const LDF &ldf, const STF &stf, const float2 *__restrict__ tri) {
    constexpr int N = 1 << L, K = pass_kind(L, P), H = pass_h(L, P);
    constexpr int R = K == KHEAD ? 8 : (K == K16 ? 16 : 4), LR = ilog2k(R), LH = ilog2k(H);
    constexpr int SC = 1 << LSC, NU = (N / R) << LSC;
    for (int u = threadIdx.x; u < NU; u += blockDim.x) {
        const int c = u & (SC - 1), v = u >> LSC;
        const int j = v & (H - 1), base = ((v >> LH) << (LH + LR)) + j;
        float2 e[R];
        ldf.template load<R, H>(e, c, base);
        if constexpr (K == KHEAD)
            math_head<INV, F>(e, tri);
        else if constexpr (K == K16)
            math16<INV, H, F>(e, tri + tw_off(L, H) + j);
        else
            math4<INV, H, F>(e, tri + tw_off(L, H) + j);
        stf.template store<R, H>(e, c, base);
    }
    __syncthreads();
}

// Passes [P, PEND) in shared memory.
template <bool INV, int L, int P, int PEND, int LSC, bool F, typename IO>
__device__ __forceinline__ void col_passes(const IO &io, const float2 *__restrict__ tri) {
    if constexpr (P < PEND) {
        col_pass<INV, L, P, LSC, F>(io, io, tri);
        col_passes<INV, L, P + 1, PEND, LSC, F>(io, tri);
    }
}

// The middle sweep (see the file header): the geometry of its units.
template <int L>
struct Mid {
    static constexpr int N = 1 << L, PL = npass(L) - 1;
    static constexpr int KL = pass_kind(L, PL), HL = pass_h(L, PL);
    static constexpr int M = ((L & 1) && KL == K4) ? 8 : 16, S = N / M;
};

// The forward cascade's last pass on x[c'] = row B + S*c' of its
// natural-order output.
template <int L>
__device__ __forceinline__ void fwd_last_pass(float2 *x, int B, const float2 *__restrict__ tri) {
    using G = Mid<L>;
    constexpr int HL = G::HL, S = G::S;
    if constexpr (G::KL == K16) {
        // one radix-16 unit at quarter S = HL, butterfly index B
        math16<false, HL>(x, tri + tw_off(L, HL) + B);
    } else if constexpr (G::M == 16) {
        // even L, radix-4 at HL = 4S: units j = B + S*q on x[q + 4i]
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float2 *t = tri + tw_off(L, HL) + B + S * q;
            bfly4<false>(&x[q], &x[q + 4], &x[q + 8], &x[q + 12], __ldg(t), __ldg(t + HL), __ldg(t + 2 * HL));
        }
    } else {
        // odd L, radix-4 at HL = 2S: units j = B, B + S on x[2i], x[2i+1]
#pragma unroll
        for (int q = 0; q < 2; q++) {
            const float2 *t = tri + tw_off(L, HL) + B + S * q;
            bfly4<false>(&x[q], &x[q + 2], &x[q + 4], &x[q + 6], __ldg(t), __ldg(t + HL), __ldg(t + 2 * HL));
        }
    }
}

// The inverse cascade's first pass on the same rows, stored through sp
// (row B + S*c' at sp[(S*c') << LSC]).
template <int L, int LSC, bool F = false>
__device__ __forceinline__ void inv_first_pass(float2 *x, float2 *sp, const float2 *__restrict__ tri) {
    using G = Mid<L>;
    constexpr int M = G::M, S = G::S;
    if constexpr (L & 1) {
        // inverse head(s): logical 8a+t <-> row B' + (N/8)*brev3(t)
#pragma unroll
        for (int hd = 0; hd < M / 8; hd++) {
            float2 e[8];
#pragma unroll
            for (int t = 0; t < 8; t++) e[t] = x[(M / 8) * brevk(t, 3) + hd];
            math_head<true, F>(e, tri);
#pragma unroll
            for (int t = 0; t < 8; t++) sp[(S * ((M / 8) * brevk(t, 3) + hd)) << LSC] = e[t];
        }
    } else {
        // inverse radix-16 at quarter 1: logical 16a+r <-> row B + S*brev4(r)
        float2 e[16];
#pragma unroll
        for (int r = 0; r < 16; r++) e[r] = x[brevk(r, 4)];
        math16<true, 1, F>(e, tri);
#pragma unroll
        for (int r = 0; r < 16; r++) sp[(S * brevk(r, 4)) << LSC] = e[r];
    }
}

// The middle sweep.  x[c'] is row B + S*c' of the forward's natural-order
// output; FWD runs the forward's last pass on it.
template <bool FWD, int L, int LSC, typename LDX, bool MUL = true, bool F = false>
__device__ __forceinline__ void middle_sweep(float2 *smem, const LDX &ldx, const float2 *__restrict__ ts, int hwp,
                                             int wv, const float2 *__restrict__ tri) {
    constexpr int M = Mid<L>::M, S = Mid<L>::S, SC = 1 << LSC;
    for (int u = threadIdx.x; u < (S << LSC); u += blockDim.x) {
        const int c = u & (SC - 1), B = u >> LSC;
        float2 x[M];
        ldx(x, c, B);
        if constexpr (FWD) fwd_last_pass<L>(x, B, tri);
        if constexpr (MUL) {
            // spec *= conj(tspec) (mulConjGo, impl.go:376-388)
            const float2 *tp = ts + (size_t)B * hwp + c;
#pragma unroll
            for (int ci = 0; ci < M; ci++)
                x[ci] = mul_conj(x[ci], c < wv ? __ldg(tp + (size_t)(S * ci) * hwp) : make_float2(0.f, 0.f));
        }
        inv_first_pass<L, LSC, F>(x, smem + (B << LSC) + c, tri);
    }
    __syncthreads();
}

// ------------------------------------------------ mode 4: fused channels
// The fast form of one colour match: every channel of a column strip in
// one CTA (channel k's [N x SC] strip at smem + k*(N << LSC)).  The
// forward passes run over all channels together, then a sweep sums each
// channel's conj-products with the zero-mean template spectra (fused
// multiply-adds) and runs the inverse's first pass once into channel 0's
// strip, then the inverse passes of that one strip.  The frame's column
// spectra never leave shared memory.

// Strip width of mode 4: 2048 / N columns (a channel strip is 16 KB).
__host__ __device__ constexpr int sc4(int L) { return (1 << L) >= 2048 ? 1 : 2048 >> L; }

template <int L, int LSC>
struct SmemNatCh {  // channel k, row r at s[k * (N << LSC) + (r << LSC) + c]
    float2 *s;
    template <int R, int STEP>
    __device__ __forceinline__ void load(float2 *e, int k, int c, int base) const {
        SmemNat<LSC>{s + ((size_t)k << (L + LSC))}.template load<R, STEP>(e, c, base);
    }
    template <int R, int STEP>
    __device__ __forceinline__ void store(const float2 *e, int k, int c, int base) const {
        SmemNat<LSC>{s + ((size_t)k << (L + LSC))}.template store<R, STEP>(e, c, base);
    }
};

template <int L>
struct GlobalSlotsCh {  // forward-rows output of channel k (see GlobalSlots)
    const float2 *src;
    size_t chanStride;
    int hwp, wv, loaded;
    template <int R, int STEP>
    __device__ __forceinline__ void load(float2 *e, int k, int c, int base) const {
        GlobalSlots<L>{src + (size_t)k * chanStride, hwp, wv, loaded}.template load<R, STEP>(e, c, base);
    }
};

// One forward pass p over channels [0, cn) of the strip.  Ends with a barrier.
template <int L, int P, int LSC, bool F, typename LDF, typename STF>
__device__ __forceinline__ void col_pass_ch(int cn, const LDF &ldf, const STF &stf, const float2 *__restrict__ tri) {
    constexpr int N = 1 << L, K = pass_kind(L, P), H = pass_h(L, P);
    constexpr int R = K == KHEAD ? 8 : (K == K16 ? 16 : 4), LR = ilog2k(R), LH = ilog2k(H);
    constexpr int SC = 1 << LSC, LNU = L - LR + LSC;
    for (int u = threadIdx.x; u < (cn << LNU); u += blockDim.x) {
        const int k = u >> LNU, w = u & ((1 << LNU) - 1);
        const int c = w & (SC - 1), v = w >> LSC;
        const int j = v & (H - 1), base = ((v >> LH) << (LH + LR)) + j;
        float2 e[R];
        ldf.template load<R, H>(e, k, c, base);
        if constexpr (K == KHEAD)
            math_head<false, F>(e, tri);
        else if constexpr (K == K16)
            math16<false, H, F>(e, tri + tw_off(L, H) + j);
        else
            math4<false, H, F>(e, tri + tw_off(L, H) + j);
        stf.template store<R, H>(e, k, c, base);
    }
    __syncthreads();
}

template <int L, int P, int PEND, int LSC, bool F>
__device__ __forceinline__ void col_passes_ch(int cn, const SmemNatCh<L, LSC> &io, const float2 *__restrict__ tri) {
    if constexpr (P < PEND) {
        col_pass_ch<L, P, LSC, F>(cn, io, io, tri);
        col_passes_ch<L, P + 1, PEND, LSC, F>(cn, io, tri);
    }
}

template <int L>
__global__ void __launch_bounds__(256, 3) k_cols_sum_t(ColsArgs a) {
    griddep_wait();
    griddep_launch();
    constexpr int N = 1 << L, NP = npass(L), SC = sc4(L), LSC = ilog2k(SC);
    constexpr int M = Mid<L>::M, S = Mid<L>::S;
    extern __shared__ float2 smem[];
    const FftClass &fc = a.fc;
    const int tileLocal = blockIdx.z;
    const int tile = fc.tileFirst + tileLocal;
    const DevMember &m = a.ms.solo;
    const DevParams &Pm = a.ms.params[m.pIdx];
    if (Pm.flat) return;
    const int cn = Pm.cn;
    const TileBox b = tile_box(a.g, tile);
    const int c0 = blockIdx.x * SC;
    const int hwp = fc.hwp;
    const int wv = min(SC, fc.hw - c0);
    const size_t chanStride = (size_t)N * hwp;
    const float2 *tri = fc.triH;
    const GlobalSlotsCh<L> gs{a.in + (size_t)tileLocal * a.cnS * chanStride + c0, chanStride, hwp, wv,
                              min(N, (b.loadH + 1) & ~1)};
    const SmemNatCh<L, LSC> sn{smem};
    // every forward pass in shared memory (the last one too: keeping it in
    // the sum sweep's registers beside the accumulator spills)
    col_pass_ch<L, 0, LSC, true>(cn, gs, sn, tri);
    col_passes_ch<L, 1, NP, LSC, true>(cn, sn, tri);
    const float2 *ts = m.tspec[a.cls] + c0;
    for (int u = threadIdx.x; u < (S << LSC); u += blockDim.x) {
        const int c = u & (SC - 1), B = u >> LSC;
        float2 acc[M];
#pragma unroll
        for (int ci = 0; ci < M; ci++) acc[ci] = make_float2(0.f, 0.f);
        for (int k = 0; k < cn; k++) {
            const float2 *p = smem + ((size_t)k << (L + LSC)) + (B << LSC) + c;
            float2 x[M];
#pragma unroll
            for (int ci = 0; ci < M; ci++) x[ci] = p[(S * ci) << LSC];
            const float2 *tp = ts + (size_t)k * chanStride + (size_t)B * hwp + c;
#pragma unroll
            for (int ci = 0; ci < M; ci++) {
                const float2 t = c < wv ? __ldg(tp + (size_t)(S * ci) * hwp) : make_float2(0.f, 0.f);
                acc[ci].x = fmaf(x[ci].x, t.x, fmaf(x[ci].y, t.y, acc[ci].x));
                acc[ci].y = fmaf(x[ci].y, t.x, fmaf(-x[ci].x, t.y, acc[ci].y));
            }
        }
        inv_first_pass<L, LSC, true>(acc, smem + (B << LSC) + c, tri);
    }
    __syncthreads();
    const int ty = tile / a.g.ntx;
    const int bh = (ty == a.g.nty - 1) ? m.rh - b.y0 : a.g.blockH;
    const SmemRev<L, LSC> sr{smem};
    const GlobalInv<L> gi{a.ms.scratch[a.cls] + (size_t)tileLocal * chanStride + c0, hwp, wv, min(N, (bh + 1) & ~1)};
    col_passes<true, L, 1, NP - 1, LSC, true>(sr, tri);
    col_pass<true, L, NP - 1, LSC, true>(sr, gi, tri);
}

template <int MODE, int L>
__global__ void __launch_bounds__(256, 3) k_cols_t(ColsArgs a) {
    griddep_wait();
    griddep_launch();
    constexpr int N = 1 << L, NP = npass(L);
    constexpr int SC = N >= 1024 ? 8192 / N : 16, LSC = ilog2k(SC);
    extern __shared__ float2 smem[];
    const FftClass &fc = a.fc;
    // modes 2 and 3 (a fleet wave): the column strip is the slowest grid
    // dimension and members vary fastest within it.  A strip partitions
    // every operand (frame tile spectra, template spectra, output), so the
    // CTAs of one strip -- all tiles x members -- touch a working set of
    // (tiles x channels + members x channels) strips, a few MB that stay in
    // L2: each frame and template spectrum leaves HBM about once per wave
    // instead of once per (member, tile) pair.
    constexpr bool WAVE = MODE >= 2;
    const int pairIdx = WAVE ? blockIdx.x : blockIdx.z;
    const int strip = WAVE ? blockIdx.z : blockIdx.x;
    const int tileLocal = WAVE ? pairIdx / a.nmem : pairIdx % fc.ntiles;
    const int slot = WAVE ? pairIdx - tileLocal * a.nmem : pairIdx / fc.ntiles;
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
    const TileBox b = tile_box(a.g, tile);
    if (WAVE && a.ms.anyRoi && roi_misses_tile(a.g, tile, b, *m)) return;  // outside the member's ROI
    const int c0 = strip * SC;
    const int hwp = fc.hwp;
    const int wv = min(SC, fc.hw - c0);
    const size_t chanStride = (size_t)N * hwp;
    const float2 *tri = fc.triH;
    const float2 *src = a.in + ((size_t)tileLocal * a.cnS + k) * chanStride + c0;
    const SmemNat<LSC> sn{smem};
    const SmemRev<L, LSC> sr{smem};
    if (!WAVE) {
        const GlobalSlots<L> gs{src, hwp, wv, min(N, (b.loadH + 1) & ~1)};
        col_pass<false, L, 0, LSC, false>(gs, sn, tri);
        if (MODE == 0) {
            col_passes<false, L, 1, NP - 1, LSC, false>(sn, tri);
            const GlobalNat gn{a.out + ((size_t)tileLocal * a.cnS + k) * chanStride + c0, hwp, wv, a.scale};
            col_pass<false, L, NP - 1, LSC, false>(sn, gn, tri);
            return;
        }
        col_passes<false, L, 1, NP - 1, LSC, false>(sn, tri);
    }
    if (MODE != 0) {
        const float2 *ts = m->tspec[a.cls] + (size_t)k * chanStride + c0;
        constexpr int PL = NP - 1;
        constexpr int M = ((L & 1) && pass_kind(L, PL) == K4) ? 8 : 16, S = N / M;
        if (MODE == 1) {
            auto ldx = [&](float2 *x, int c, int B) {
                const float2 *p = smem + (B << LSC) + c;
#pragma unroll
                for (int ci = 0; ci < M; ci++) x[ci] = p[(S * ci) << LSC];
            };
            middle_sweep<true, L, LSC>(smem, ldx, ts, hwp, wv, tri);
        } else if (MODE == 2) {
            // the frame tile's stored natural-order spectrum
            auto ldx = [&](float2 *x, int c, int B) {
                const float2 *p = src + (size_t)B * hwp + c;
#pragma unroll
                for (int ci = 0; ci < M; ci++) x[ci] = c < wv ? __ldg(p + (size_t)(S * ci) * hwp) : make_float2(0.f, 0.f);
            };
            middle_sweep<false, L, LSC>(smem, ldx, ts, hwp, wv, tri);
        } else {
            // Mode 3 (the fast form) sums over the member's channels frame x
            // conj(zero-mean template) from stored spectra, straight into the
            // registers of the inverse's first pass.  (A version that staged
            // the sum into the strip first measured 3.63 against 3.50 ms per
            // 256-member 2560x1440 frame: the strip's extra store and load
            // are shared-memory traffic in a kernel bound by it.)
            const float2 *fr = a.in + (size_t)tileLocal * a.cnS * chanStride + c0;
            const float2 *tq = m->tspec[a.cls] + c0;
            // The channel sum formed in the registers of the inverse's first
            // pass: each unit's M rows of every channel come from the stored
            // spectra (32-bit element offsets from each channel's base), so
            // the sum makes no round trip through shared memory.
            const unsigned sStep = (unsigned)(S * hwp);
            auto ldx = [&](float2 *x, int c, int B) {
#pragma unroll
                for (int ci = 0; ci < M; ci++) x[ci] = make_float2(0.f, 0.f);
                if (c >= wv) return;
                const unsigned o0 = (unsigned)(B * hwp + c);
                auto chan = [&](int kk) {
                    const float2 *fk = fr + (size_t)kk * chanStride, *tk = tq + (size_t)kk * chanStride;
                    // eight rows' loads in flight at a time (16 would spill)
#pragma unroll
                    for (int h = 0; h < M; h += 8) {
                        float2 f[8], t[8];
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            f[i] = __ldg(fk + (o0 + (unsigned)(h + i) * sStep));
                            t[i] = __ldg(tk + (o0 + (unsigned)(h + i) * sStep));
                        }
#pragma unroll
                        for (int i = 0; i < 8; i++) {
                            float2 &xi = x[h + i];
                            xi.x = fmaf(f[i].x, t[i].x, fmaf(f[i].y, t[i].y, xi.x));
                            xi.y = fmaf(f[i].y, t[i].x, fmaf(-f[i].x, t[i].y, xi.y));
                        }
                    }
                };
                if (cn == 3) {
                    chan(0);
                    chan(1);
                    chan(2);
                } else {
                    for (int kk = 0; kk < cn; kk++) chan(kk);
                }
            };
            middle_sweep<false, L, LSC, decltype(ldx), false, true>(smem, ldx, nullptr, hwp, wv, tri);
        }
        const int ty = tile / a.g.ntx;
        const int bh = (ty == a.g.nty - 1) ? m->rh - b.y0 : a.g.blockH;
        const size_t scrOff = MODE == 3 ? (size_t)tileLocal * chanStride : ((size_t)tileLocal * a.cnS + k) * chanStride;
        const GlobalInv<L> gi{a.ms.scratch[a.cls] + (size_t)slot * a.ms.scratchStride[a.cls] + scrOff + c0, hwp, wv,
                              min(N, (bh + 1) & ~1)};
        col_passes<true, L, 1, NP - 1, LSC, MODE == 3>(sr, tri);
        col_pass<true, L, NP - 1, LSC, MODE == 3>(sr, gi, tri);
    }
}

template <int MODE, int L>
void cols_one(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    set_smem(k_cols_t<MODE, L>, smem);
    launch_k(k_cols_t<MODE, L>, grid, dim3(kThreads), smem, st, a);
}

template <int L>
void cols_sum_one(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    set_smem(k_cols_sum_t<L>, smem);
    launch_k(k_cols_sum_t<L>, grid, dim3(kThreads), smem, st, a);
}

template <int MODE>
void cols_mode(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    switch (a.fc.log2H) {
        case 5: cols_one<MODE, 5>(a, grid, smem, st); break;
        case 6: cols_one<MODE, 6>(a, grid, smem, st); break;
        case 7: cols_one<MODE, 7>(a, grid, smem, st); break;
        case 8: cols_one<MODE, 8>(a, grid, smem, st); break;
        case 9: cols_one<MODE, 9>(a, grid, smem, st); break;
        case 10: cols_one<MODE, 10>(a, grid, smem, st); break;
        case 11: cols_one<MODE, 11>(a, grid, smem, st); break;
        default: cols_one<MODE, 12>(a, grid, smem, st); break;
    }
}

}  // namespace

bool cols_fixed_length(int log2H) { return log2H >= 5 && log2H <= 12; }

int cols_sum_width(int log2H) { return sc4(log2H); }

void launch_cols_sum(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    switch (a.fc.log2H) {
        case 5: cols_sum_one<5>(a, grid, smem, st); break;
        case 6: cols_sum_one<6>(a, grid, smem, st); break;
        case 7: cols_sum_one<7>(a, grid, smem, st); break;
        case 8: cols_sum_one<8>(a, grid, smem, st); break;
        case 9: cols_sum_one<9>(a, grid, smem, st); break;
        case 10: cols_sum_one<10>(a, grid, smem, st); break;
        case 11: cols_sum_one<11>(a, grid, smem, st); break;
        default: cols_sum_one<12>(a, grid, smem, st); break;
    }
}

void launch_cols_fixed(const ColsArgs &a, dim3 grid, size_t smem, cudaStream_t st) {
    if (a.mode == 0)
        cols_mode<0>(a, grid, smem, st);
    else if (a.mode == 1)
        cols_mode<1>(a, grid, smem, st);
    else if (a.mode == 2)
        cols_mode<2>(a, grid, smem, st);
    else
        cols_mode<3>(a, grid, smem, st);
}

}  // namespace cvm
