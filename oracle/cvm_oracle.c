/*
 * cvm_oracle.c -- CPU restatement of cvmatch's TM_CCOEFF_NORMED path.
 *
 * TEST INFRASTRUCTURE ONLY (see cvm_oracle.h).  Compile with
 * -O2 -ffp-contract=off and without fast-math: every float expression
 * below must round once per operation, exactly like the reference's
 * pinned Go sequence (radix4.go:17-32, impl.go:816-849).
 *
 * Each function names the reference file:line it restates.  The
 * scheduling of the reference (worker teams, chunked spills, SIMD
 * kernels) is pure scheduling that never changes a bit
 * (impl_simd_test.go:26-66, threads_test.go:62-81), so this file follows
 * the scalar per-element arithmetic and schedules work in its own way.
 */
#include "cvm_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct { float re, im; } cf;

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

static int next_pow2(int v) {
    int n = 1;
    while (n < v) n <<= 1;
    return n;
}

static int ilog2(int n) { /* n a power of two */
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

/* oddLog2 (radix4.go:37): bits.Len(n) even  <=>  log2(n) odd. */
static int odd_log2(int n) { return ilog2(n) & 1; }

/* ------------------------------------------------------------ twiddles */

/* sincospiFrac, impl.go:98-133: dyadic range reduction and the fdlibm
 * kernel polynomials, every product rounded before it is added. */
void cvo_sincospi(int j, int half, float *c_out, float *s_out) {
    int m = 2 * j;
    int k = m / half;
    int rem = m - k * half;
    double u = (double)rem / (double)half;
    int swap = 0;
    if (u > 0.5) {
        u = 1.0 - u;
        swap = 1;
    }
    double y = u * 1.57079632679489661923;
    double z = y * y;
    double t;
    t = z * -1.13596475577881948265e-11;
    t = z * (2.08757232129817482790e-09 + t);
    t = z * (-2.75573143513906633035e-07 + t);
    t = z * (2.48015872894767294178e-05 + t);
    t = z * (-1.38888888888741095749e-03 + t);
    double r = z * (4.16666666666666019037e-02 + t);
    double hz = 0.5 * z;
    double w = 1.0 - hz;
    double zr = z * r;
    double c = w + (((1.0 - w) - hz) + zr);
    double q;
    q = z * 1.58969099521155010221e-10;
    q = z * (-2.50507602534068634195e-08 + q);
    q = z * (2.75573137070700676789e-06 + q);
    q = z * (-1.98412698298579493134e-04 + q);
    double r2 = 8.33333333332248946124e-03 + q;
    double v = z * y;
    double zr2 = z * r2;
    double s = y + v * (-1.66666666666666324348e-01 + zr2);
    if (swap) {
        double tmp = c;
        c = s;
        s = tmp;
    }
    if (k != 0) {
        double tmp = c;
        c = -s;
        s = tmp;
    }
    *c_out = (float)c;
    *s_out = (float)s;
}

/* makeTriTwiddles, radix4.go:45-73. */
int cvo_tri_twiddles(int n, float *tri) {
    int cnt = 0;
    int h = odd_log2(n) ? 2 : 1;
    for (; 4 * h <= n; h *= 4) {
        for (int j = 0; j < h; j++) {
            float c, s;
            cvo_sincospi(j, 2 * h, &c, &s);
            if (tri) { tri[2 * cnt] = c; tri[2 * cnt + 1] = -s; }
            cnt++;
        }
        for (int j = 0; j < h; j++) {
            float c, s;
            cvo_sincospi(j, h, &c, &s);
            if (tri) { tri[2 * cnt] = c; tri[2 * cnt + 1] = -s; }
            cnt++;
        }
        for (int j = 0; j < h; j++) {
            int m = 3 * j, neg = 0;
            if (m >= 2 * h) { m -= 2 * h; neg = 1; }
            float c, s;
            cvo_sincospi(m, 2 * h, &c, &s);
            if (neg) { c = -c; s = -s; }
            if (tri) { tri[2 * cnt] = c; tri[2 * cnt + 1] = -s; }
            cnt++;
        }
    }
    return cnt;
}

/* Per-size tables (fftTables, impl.go:148-208). */
typedef struct {
    int n;
    cf *tri;
    int32_t *brev;
} tab_t;

static pthread_mutex_t tab_mu = PTHREAD_MUTEX_INITIALIZER;
static tab_t *tabs[31];

static const tab_t *tables(int n) {
    int l = ilog2(n);
    pthread_mutex_lock(&tab_mu);
    tab_t *t = tabs[l];
    if (!t) {
        t = (tab_t *)calloc(1, sizeof(tab_t));
        t->n = n;
        int cnt = cvo_tri_twiddles(n, NULL);
        t->tri = (cf *)malloc(sizeof(cf) * (size_t)(cnt > 0 ? cnt : 1));
        cvo_tri_twiddles(n, (float *)t->tri);
        /* makeBitrev, impl.go:148-165 */
        t->brev = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
        int br = 0;
        for (int i = 0; i < n; i++) {
            t->brev[i] = br;
            int bit = n >> 1;
            while (br & bit) {
                br ^= bit;
                bit >>= 1;
            }
            br |= bit;
        }
        tabs[l] = t;
    }
    pthread_mutex_unlock(&tab_mu);
    return t;
}

/* --------------------------------------------------------- FFT engine */

/* mulPlain, radix4.go:80-85. */
static inline cf mulp(cf v, cf w) {
    float a = v.re * w.re, b = v.im * w.im;
    float c = v.re * w.im, d = v.im * w.re;
    cf r = {a - b, c + d};
    return r;
}

/* One radix-4 butterfly on (A at r, C at r+h, B at r+2h, D at r+3h),
 * radix4.go:126-147 (and radix4cols.go:77-101). */
static inline void bfly4(cf *pa, cf *pc, cf *pb, cf *pd, cf bw, cf cw, cf dw, int inverse) {
    if (inverse) {
        bw.im = -bw.im;
        cw.im = -cw.im;
        dw.im = -dw.im;
    }
    cf av = *pa;
    cf tb = mulp(*pb, bw);
    cf tc = mulp(*pc, cw);
    cf td = mulp(*pd, dw);
    cf s0 = {av.re + tc.re, av.im + tc.im};
    cf s1 = {av.re - tc.re, av.im - tc.im};
    cf s2 = {tb.re + td.re, tb.im + td.im};
    cf s3 = {tb.re - td.re, tb.im - td.im};
    float rr, ri;
    if (inverse) { rr = -s3.im; ri = s3.re; }
    else { rr = s3.im; ri = -s3.re; }
    pa->re = s0.re + s2.re; pa->im = s0.im + s2.im;
    pc->re = s1.re + rr;    pc->im = s1.im + ri;
    pb->re = s0.re - s2.re; pb->im = s0.im - s2.im;
    pd->re = s1.re - rr;    pd->im = s1.im - ri;
}

/* fftR4 + fftR4Scalar, radix4.go:91-149. */
static void fft_r4(cf *a, int n, const tab_t *t, int inverse) {
    for (int i = 0; i < n; i++) {
        int j = t->brev[i];
        if (i < j) { cf x = a[i]; a[i] = a[j]; a[j] = x; }
    }
    int h = 1;
    if (odd_log2(n)) {
        for (int i = 0; i < n; i += 2) {
            cf u = a[i], v = a[i + 1];
            a[i].re = u.re + v.re; a[i].im = u.im + v.im;
            a[i + 1].re = u.re - v.re; a[i + 1].im = u.im - v.im;
        }
        h = 2;
    }
    const cf *tri = t->tri;
    for (; 4 * h <= n; h *= 4) {
        const cf *w1 = tri, *w2 = tri + h, *w3 = tri + 2 * h;
        tri += 3 * h;
        for (int base = 0; base < n; base += 4 * h)
            for (int j = 0; j < h; j++)
                bfly4(&a[base + j], &a[base + j + h], &a[base + j + 2 * h], &a[base + j + 3 * h],
                      w1[j], w2[j], w3[j], inverse);
    }
}

void cvo_fft_r4(float *a, int n, int inverse) { fft_r4((cf *)a, n, tables(n), inverse); }

/* colsR4Go, radix4cols.go:35-125: the row engine's sequence applied to
 * every column; rmap conjugates row access by the bit reversal. */
static void cols_r4(cf *d, int n, int width, const tab_t *t, int inverse, const int32_t *rmap) {
    int h = 1;
    if (odd_log2(n)) {
        for (int r = 0; r < n; r += 2) {
            int i0 = r, i1 = r + 1;
            if (rmap) { i0 = rmap[i0]; i1 = rmap[i1]; }
            cf *p = d + (size_t)i0 * width, *q = d + (size_t)i1 * width;
            for (int c = 0; c < width; c++) {
                cf u = p[c], v = q[c];
                p[c].re = u.re + v.re; p[c].im = u.im + v.im;
                q[c].re = u.re - v.re; q[c].im = u.im - v.im;
            }
        }
        h = 2;
    }
    const cf *tri = t->tri;
    for (; 4 * h <= n; h *= 4) {
        const cf *w1 = tri, *w2 = tri + h, *w3 = tri + 2 * h;
        tri += 3 * h;
        for (int base = 0; base < n; base += 4 * h) {
            for (int j = 0; j < h; j++) {
                int r = base + j;
                int i0 = r, i1 = r + h, i2 = r + 2 * h, i3 = r + 3 * h;
                if (rmap) { i0 = rmap[i0]; i1 = rmap[i1]; i2 = rmap[i2]; i3 = rmap[i3]; }
                cf *pA = d + (size_t)i0 * width, *pC = d + (size_t)i1 * width;
                cf *pB = d + (size_t)i2 * width, *pD = d + (size_t)i3 * width;
                for (int c = 0; c < width; c++)
                    bfly4(&pA[c], &pC[c], &pB[c], &pD[c], w1[j], w2[j], w3[j], inverse);
            }
        }
    }
}

void cvo_cols_r4(float *d, int n, int width, int inverse, int use_rmap) {
    const tab_t *t = tables(n);
    cols_r4((cf *)d, n, width, t, inverse, use_rmap ? t->brev : NULL);
}

/* ---------------------------------------------------------------- plan */

typedef struct {
    int dftW, dftH, hw, blockW, blockH;
    int64_t cost;
    const tab_t *tW, *tH;
} plan_t;

/* newGoPlan, impl.go:246-295. */
static void plan_make(int tw, int th, int rw, int rh, plan_t *p) {
    const int64_t areaCap = (int64_t)1 << 22;
    int minW = imax(2, next_pow2(tw)), minH = imax(2, next_pow2(th));
    int maxW = imax(minW, next_pow2(rw + tw - 1)), maxH = imax(minH, next_pow2(rh + th - 1));
    int bestW = minW, bestH = minH;
    int64_t bestCost = -1, bestArea = 0;
    for (int dW = minW; dW <= maxW; dW <<= 1) {
        for (int dH = minH; dH <= maxH; dH <<= 1) {
            int64_t area = (int64_t)dW * dH;
            if (area > areaCap) continue;
            int bW = imin(dW - tw + 1, rw), bH = imin(dH - th + 1, rh);
            int64_t ntx = (rw + bW - 1) / bW;
            int64_t hw = dW / 2 + 1;
            int64_t rowFFT = 5 * (int64_t)dW * ilog2(dW);
            int64_t colPass = 5 * (int64_t)dH * ilog2(dH) * hw;
            int64_t specN = (int64_t)dH * hw;
            int64_t cost = 0;
            for (int y0 = 0; y0 < rh; y0 += bH) {
                int bh = imin(bH, rh - y0);
                int loadH = imin(bh + th - 1, dH);
                cost += ntx * ((int64_t)((loadH + 1) / 2 + (bh + 1) / 2) * rowFFT + 2 * colPass + 16 * specN);
            }
            if (bestCost < 0 || cost < bestCost || (cost == bestCost && area < bestArea)) {
                bestCost = cost; bestArea = area; bestW = dW; bestH = dH;
            }
        }
    }
    p->dftW = bestW;
    p->dftH = bestH;
    p->hw = bestW / 2 + 1;
    p->cost = bestCost;
    p->blockW = imin(bestW - tw + 1, rw);
    p->blockH = imin(bestH - th + 1, rh);
    p->tW = NULL;
    p->tH = NULL;
}

static void plan_tables(plan_t *p) {
    p->tW = tables(p->dftW);
    p->tH = tables(p->dftH);
}

void cvo_plan_make(int tw, int th, int rw, int rh, cvo_plan *out) {
    plan_t p;
    plan_make(tw, th, rw, rh, &p);
    out->dft_w = p.dftW; out->dft_h = p.dftH; out->hw = p.hw;
    out->block_w = p.blockW; out->block_h = p.blockH; out->cost = p.cost;
}

/* shrinkDH, impl.go:573-582. */
static int shrink_dh(const plan_t *p, int rh, int th) {
    int lastY0 = ((rh - 1) / p->blockH) * p->blockH;
    int lastBh = rh - lastY0;
    if (lastY0 > 0) {
        int dh2 = imax(2, next_pow2(lastBh + th - 1));
        if (dh2 < p->dftH) return dh2;
    }
    return 0;
}

int cvo_shrink_dh(const cvo_plan *q, int rh, int th) {
    plan_t p;
    memset(&p, 0, sizeof p);
    p.dftH = q->dft_h; p.blockH = q->block_h;
    return shrink_dh(&p, rh, th);
}

int64_t cvo_stats_cap(int cn) {
    static const int64_t caps[5] = {0, 11909805, 8421504, 6876129, 5954902};
    return (cn >= 1 && cn <= 4) ? caps[cn] : 0;
}

/* ------------------------------------------------------- tile pipeline */

/* forwardRowPair, impl.go:301-344 (scalar branches). */
static void forward_row_pair(const uint8_t *chan, int64_t stride, int step, int x0, int y0,
                             int loadW, int loadH, const plan_t *p, cf *spec, cf *z, int r) {
    int n = p->dftW, hw = p->hw, mask = n - 1;
    cf *sa = spec + (size_t)p->tH->brev[r] * hw;
    cf *sb = spec + (size_t)p->tH->brev[r + 1] * hw;
    const uint8_t *ra = chan + (int64_t)(y0 + r) * stride + (int64_t)x0 * step;
    if (r + 1 < loadH) {
        const uint8_t *rb = chan + (int64_t)(y0 + r + 1) * stride + (int64_t)x0 * step;
        for (int x = 0; x < loadW; x++) { z[x].re = (float)ra[x * step]; z[x].im = (float)rb[x * step]; }
    } else {
        for (int x = 0; x < loadW; x++) { z[x].re = (float)ra[x * step]; z[x].im = 0.0f; }
    }
    for (int x = loadW; x < n; x++) { z[x].re = 0.0f; z[x].im = 0.0f; }
    fft_r4(z, n, p->tW, 0);
    for (int k = 0; k < hw; k++) {
        cf zk = z[k], zn = z[(n - k) & mask];
        sa[k].re = 0.5f * (zk.re + zn.re);
        sa[k].im = 0.5f * (zk.im - zn.im);
        sb[k].re = 0.5f * (zk.im + zn.im);
        sb[k].im = 0.5f * (zn.re - zk.re);
    }
}

/* blockForwardGo, impl.go:350-374. */
static void block_forward(const uint8_t *chan, int64_t stride, int step, int x0, int y0,
                          int loadW, int loadH, const plan_t *p, cf *spec, cf *z) {
    int hw = p->hw;
    int loaded = imin(p->dftH, (loadH + 1) & ~1);
    for (int r = loaded; r < p->dftH; r++)
        memset(spec + (size_t)p->tH->brev[r] * hw, 0, sizeof(cf) * (size_t)hw);
    for (int r = 0; r < loadH && r < p->dftH; r += 2)
        forward_row_pair(chan, stride, step, x0, y0, loadW, loadH, p, spec, z, r);
    cols_r4(spec, p->dftH, hw, p->tH, 0, NULL);
}

/* mulConjGo, impl.go:376-388. */
static void mul_conj(cf *spec, const cf *ts, size_t n) {
    for (size_t i = 0; i < n; i++) {
        cf a = spec[i], b = ts[i];
        float p0 = a.re * b.re, p1 = a.im * b.im;
        float p2 = a.im * b.re, p3 = a.re * b.im;
        spec[i].re = p0 + p1;
        spec[i].im = p2 - p3;
    }
}

/* inverseRowPair, impl.go:394-444 (scalar branches). */
static void inverse_row_pair(const plan_t *p, cf *spec, cf *z, float *res, int rw, int x0, int y0,
                             int bw, int bh, int add, int r) {
    int n = p->dftW, hw = p->hw;
    const cf *sa = spec + (size_t)p->tH->brev[r] * hw;
    const cf *sb = spec + (size_t)p->tH->brev[r + 1] * hw;
    for (int k = 0; k < hw; k++) {
        z[k].re = sa[k].re - sb[k].im;
        z[k].im = sa[k].im + sb[k].re;
    }
    for (int k = hw; k < n; k++) {
        int m = n - k;
        z[k].re = sa[m].re + sb[m].im;
        z[k].im = sb[m].re - sa[m].im;
    }
    fft_r4(z, n, p->tW, 1);
    float *o = res + (size_t)(y0 + r) * rw + x0;
    float *o2 = (r + 1 < bh) ? res + (size_t)(y0 + r + 1) * rw + x0 : NULL;
    if (add) {
        for (int x = 0; x < bw; x++) o[x] += z[x].re;
        if (o2) for (int x = 0; x < bw; x++) o2[x] += z[x].im;
    } else {
        for (int x = 0; x < bw; x++) o[x] = z[x].re;
        if (o2) for (int x = 0; x < bw; x++) o2[x] = z[x].im;
    }
}

/* blockInverseEmitGo, impl.go:446-464. */
static void block_inverse_emit(const plan_t *p, cf *spec, cf *z, float *res, int rw, int x0, int y0,
                               int bw, int bh, int add) {
    cols_r4(spec, p->dftH, p->hw, p->tH, 1, p->tH->brev);
    for (int r = 0; r < bh; r += 2) inverse_row_pair(p, spec, z, res, rw, x0, y0, bw, bh, add, r);
}

/* tspecSet, impl.go:484-561: template spectra on plan p, plus the
 * shrunk last-band plan and its gathered spectrum (shrinkInto,
 * impl.go:591-610). */
typedef struct {
    cf *spec;
    int has2;
    plan_t p2;
    cf *spec2;
} tset_t;

static void tset_build(const uint8_t *tpl, int64_t tstride, int step, int cn, int tw, int th, int rh,
                       int shrinkTH, const plan_t *p, tset_t *s) {
    size_t specN = (size_t)p->dftH * p->hw;
    s->spec = (cf *)malloc(sizeof(cf) * (size_t)cn * specN);
    cf *z = (cf *)malloc(sizeof(cf) * (size_t)p->dftW);
    float scale = 1.0f / ((float)p->dftW * (float)p->dftH);
    for (int k = 0; k < cn; k++) {
        cf *ts = s->spec + (size_t)k * specN;
        block_forward(tpl + k, tstride, step, 0, 0, tw, th, p, ts, z);
        for (size_t i = 0; i < specN; i++) {
            ts[i].re = ts[i].re * scale;
            ts[i].im = ts[i].im * scale;
        }
    }
    free(z);
    s->has2 = 0;
    s->spec2 = NULL;
    int dh2 = shrink_dh(p, rh, shrinkTH);
    if (dh2 > 0) {
        s->has2 = 1;
        s->p2 = *p;
        s->p2.dftH = dh2;
        s->p2.tH = tables(dh2);
        int shift = ilog2(p->dftH) - ilog2(dh2);
        float up = (float)(1 << shift);
        s->spec2 = (cf *)malloc(sizeof(cf) * (size_t)cn * dh2 * p->hw);
        for (int k = 0; k < cn; k++)
            for (int r = 0; r < dh2; r++) {
                const cf *src = s->spec + (size_t)k * specN + (size_t)(r << shift) * p->hw;
                cf *dst = s->spec2 + ((size_t)k * dh2 + r) * p->hw;
                for (int x = 0; x < p->hw; x++) {
                    dst[x].re = src[x].re * up;
                    dst[x].im = src[x].im * up;
                }
            }
    }
}

static void tset_free(tset_t *s) {
    free(s->spec);
    free(s->spec2);
}

/* ------------------------------------------------------------- threads */

typedef void (*work_fn)(void *ctx, int w);
typedef struct { work_fn fn; void *ctx; int w; } thr_arg;

static void *thr_main(void *a) {
    thr_arg *t = (thr_arg *)a;
    t->fn(t->ctx, t->w);
    return NULL;
}

/* runParallel, impl.go:72-87. */
static void run_parallel(int n, work_fn fn, void *ctx) {
    if (n <= 1) { fn(ctx, 0); return; }
    pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)n);
    thr_arg *args = (thr_arg *)malloc(sizeof(thr_arg) * (size_t)n);
    for (int i = 1; i < n; i++) {
        args[i].fn = fn; args[i].ctx = ctx; args[i].w = i;
        pthread_create(&th[i], NULL, thr_main, &args[i]);
    }
    fn(ctx, 0);
    for (int i = 1; i < n; i++) pthread_join(th[i], NULL);
    free(th);
    free(args);
}

static int clamp_threads(int n) { return n < 1 ? 1 : (n > 16 ? 16 : n); }

/* ------------------------------------------------------ crossCorrGo */

typedef struct {
    const uint8_t *img;
    int64_t istride;
    int step, cn, tw, th, rw, rh;
    const plan_t *p;
    const tset_t *set;
    float *res;
    int ntx, ntiles, lastY0;
    atomic_int next;
} cc_ctx;

static void cc_worker(void *vctx, int w) {
    (void)w;
    cc_ctx *c = (cc_ctx *)vctx;
    const plan_t *p = c->p;
    size_t specN = (size_t)p->dftH * p->hw;
    cf *spec = (cf *)malloc(sizeof(cf) * specN);
    cf *z = (cf *)malloc(sizeof(cf) * (size_t)p->dftW);
    for (;;) {
        int t = atomic_fetch_add(&c->next, 1);
        if (t >= c->ntiles) break;
        int x0 = (t % c->ntx) * p->blockW, y0 = (t / c->ntx) * p->blockH;
        int bw = imin(p->blockW, c->rw - x0), bh = imin(p->blockH, c->rh - y0);
        const plan_t *bp = p;
        const cf *bt = c->set->spec;
        if (y0 == c->lastY0 && c->set->has2) { bp = &c->set->p2; bt = c->set->spec2; }
        size_t sn = (size_t)bp->dftH * bp->hw;
        for (int k = 0; k < c->cn; k++) {
            block_forward(c->img + k, c->istride, c->step, x0, y0, bw + c->tw - 1, bh + c->th - 1, bp, spec, z);
            mul_conj(spec, bt + (size_t)k * sn, sn);
            block_inverse_emit(bp, spec, z, c->res, c->rw, x0, y0, bw, bh, k > 0);
        }
    }
    free(spec);
    free(z);
}

/* crossCorrGo, impl.go:616-693. */
static void cross_corr(const uint8_t *img, int64_t istride, int step, int cn, int tw, int th, int rw,
                       int rh, int threads, const plan_t *p, const tset_t *set, float *res) {
    cc_ctx c;
    c.img = img; c.istride = istride; c.step = step; c.cn = cn; c.tw = tw; c.th = th;
    c.rw = rw; c.rh = rh; c.p = p; c.set = set; c.res = res;
    c.ntx = (rw + p->blockW - 1) / p->blockW;
    int nty = (rh + p->blockH - 1) / p->blockH;
    c.ntiles = c.ntx * nty;
    c.lastY0 = ((rh - 1) / p->blockH) * p->blockH;
    atomic_init(&c.next, 0);
    run_parallel(imin(threads, c.ntiles), cc_worker, &c);
}

/* ------------------------------------------------ normalization + scan */

/* normOne, impl.go:825-849. */
static inline float norm_one(float num, float lane0, float idiff, float s2, float numScale,
                             float varScale, float eps, float templNorm) {
    float t = lane0 * numScale;
    num = num - t;
    float diff2 = idiff * varScale;
    float lim = eps * s2;
    if (lim > 0.5f) lim = 0.5f;
    float den = 0.0f;
    if (diff2 > lim) {
        float sq = (float)sqrt((double)diff2);
        den = sq * templNorm;
    }
    float band = den * 1.125f;
    if (fabsf(num) < den) num = num / den;
    else if (fabsf(num) < band) num = num > 0.0f ? 1.0f : -1.0f;
    else num = 0.0f;
    return num;
}

/* float32(float64(v)) for an int64: the reference's two-step conversion
 * (double rounding above 2^53 is part of the pinned sequence). */
static float f32_via_f64(int64_t v) {
    volatile double d = (double)v;
    return (float)d;
}

typedef struct {
    float minV, maxV;
    int minX, minY, maxX, maxY;
} ext_t;

/* normalizeBandGo, impl.go:859-1054 (colBuildGo/colSlideGo 708-805). */
static ext_t normalize_band(const uint8_t *img, int64_t istride, int iw, int cn, int step, int tw,
                            int th, int rw, int y0, int y1, const int64_t *tsum, float templNorm,
                            const float *corr, float *result) {
    int64_t area = (int64_t)tw * th;
    float varScale = (float)(1.0 / ((double)tw * (double)th));
    float numScale = varScale;
    if (cn == 1) numScale = (float)((double)tsum[0] / ((double)tw * (double)th));
    int cs = (step == 4 && (cn == 3 || cn == 4)) ? 4 : cn;
    int32_t *colSum = (int32_t *)calloc((size_t)iw * cs, sizeof(int32_t));
    int64_t *colSum2 = (int64_t *)calloc((size_t)iw, sizeof(int64_t));
    for (int y = y0; y < y0 + th; y++) {
        const uint8_t *row = img + (int64_t)y * istride;
        for (int x = 0; x < iw; x++) {
            int64_t q = 0;
            for (int k = 0; k < cn; k++) {
                int32_t v = row[x * step + k];
                colSum[x * cs + k] += v;
                q += v * v;
            }
            colSum2[x] += q;
        }
    }
    ext_t e;
    e.minV = FLT_MAX; e.maxV = -FLT_MAX;
    e.minX = 0; e.minY = y0; e.maxX = 0; e.maxY = y0;
    const float eps = (float)(10.0 * 0x1p-23);
    for (int y = y0;; y++) {
        int64_t s[4] = {0, 0, 0, 0}, s2 = 0;
        for (int x = 0; x < tw; x++) {
            for (int k = 0; k < cn; k++) s[k] += colSum[x * cs + k];
            s2 += colSum2[x];
        }
        float *rrow = result + (size_t)y * rw;
        const float *crow = corr + (size_t)y * rw;
        for (int x = 0; x < rw; x++) {
            int64_t lane0 = 0, sq = 0;
            for (int k = 0; k < cn; k++) {
                lane0 += s[k] * tsum[k];
                sq += s[k] * s[k];
            }
            if (cn == 1) lane0 = s[0];
            float l0 = f32_via_f64(lane0);
            float id = f32_via_f64(area * s2 - sq);
            float q2 = f32_via_f64(s2);
            rrow[x] = norm_one(crow[x], l0, id, q2, numScale, varScale, eps, templNorm);
            if (x + 1 < rw) {
                for (int k = 0; k < cn; k++) s[k] += (int64_t)(colSum[(x + tw) * cs + k] - colSum[x * cs + k]);
                s2 += colSum2[x + tw] - colSum2[x];
            }
        }
        for (int x = 0; x < rw; x++) {
            float v = rrow[x];
            if (v < e.minV) { e.minV = v; e.minX = x; e.minY = y; }
            if (v > e.maxV) { e.maxV = v; e.maxX = x; e.maxY = y; }
        }
        if (y + 1 >= y1) break;
        const uint8_t *rsub = img + (int64_t)y * istride, *radd = img + (int64_t)(y + th) * istride;
        for (int x = 0; x < iw; x++) {
            int64_t dq = 0;
            for (int k = 0; k < cn; k++) {
                int32_t a = radd[x * step + k], b = rsub[x * step + k];
                colSum[x * cs + k] += a - b;
                dq += a * a - b * b;
            }
            colSum2[x] += dq;
        }
    }
    free(colSum);
    free(colSum2);
    return e;
}

typedef struct {
    const uint8_t *img;
    int64_t istride;
    int iw, cn, step, tw, th, rw;
    const int *bandY;
    const int64_t *tsum;
    float templNorm;
    const float *corr;
    float *result;
    ext_t *ext;
} nb_ctx;

static void nb_worker(void *vctx, int w) {
    nb_ctx *c = (nb_ctx *)vctx;
    c->ext[w] = normalize_band(c->img, c->istride, c->iw, c->cn, c->step, c->tw, c->th, c->rw,
                               c->bandY[w], c->bandY[w + 1], c->tsum, c->templNorm, c->corr, c->result);
}

/* normalizeParallelGo, impl.go:1081-1114. */
static void normalize_parallel(const uint8_t *img, int64_t istride, int iw, int tw, int th, int cn,
                               int step, int rw, int rh, int threads, const int64_t *tsum,
                               int64_t varSum, const float *corr, float *result, cvo_result *out) {
    float templNorm = (float)sqrt((double)varSum / ((double)tw * (double)th));
    int nb = threads;
    int maxb = rh / imax(th, 32);
    if (maxb >= 1 && nb > maxb) nb = maxb;
    nb = imax(imin(nb, rh), 1);
    int *bandY = (int *)malloc(sizeof(int) * (size_t)(nb + 1));
    for (int b = 0; b <= nb; b++) bandY[b] = (int)((int64_t)rh * b / nb);
    ext_t *ext = (ext_t *)malloc(sizeof(ext_t) * (size_t)nb);
    nb_ctx c = {img, istride, iw, cn, step, tw, th, rw, bandY, tsum, templNorm, corr, result, ext};
    run_parallel(nb, nb_worker, &c);
    ext_t r = ext[0];
    for (int b = 1; b < nb; b++) {
        if (ext[b].minV < r.minV) { r.minV = ext[b].minV; r.minX = ext[b].minX; r.minY = ext[b].minY; }
        if (ext[b].maxV > r.maxV) { r.maxV = ext[b].maxV; r.maxX = ext[b].maxX; r.maxY = ext[b].maxY; }
    }
    out->min_v = r.minV; out->min_x = r.minX; out->min_y = r.minY;
    out->max_v = r.maxV; out->max_x = r.maxX; out->max_y = r.maxY;
    free(bandY);
    free(ext);
}

void cvo_normalize(const uint8_t *img, int64_t istride, int iw, int ih, int tw, int th, int cn,
                   int step, const int64_t tsum[4], int64_t var_sum, int threads, const float *corr,
                   float *result, cvo_result *out) {
    (void)ih;
    normalize_parallel(img, istride, iw, tw, th, cn, step, iw - tw + 1, ih - th + 1,
                       clamp_threads(threads), tsum, var_sum, corr, result, out);
}

/* --------------------------------------------------------- entry point */

/* templStats, impl.go:1063-1079. */
void cvo_templ_stats(const uint8_t *tpl, int64_t tstride, int tw, int th, int cn, int step,
                     int64_t tsum[4], int64_t *var_sum) {
    int64_t area = (int64_t)tw * th;
    *var_sum = 0;
    for (int k = 0; k < 4; k++) tsum[k] = 0;
    for (int k = 0; k < cn; k++) {
        int64_t s = 0, s2 = 0;
        for (int y = 0; y < th; y++) {
            const uint8_t *row = tpl + (int64_t)y * tstride + k;
            for (int x = 0; x < tw; x++) {
                int64_t v = row[x * step];
                s += v;
                s2 += v * v;
            }
        }
        tsum[k] = s;
        *var_sum += area * s2 - s * s;
    }
}

static int check_args(int iw, int ih, int64_t istride, int64_t tstride, int tw, int th, int cn,
                      int step, char *err) {
    if (cn < 1 || cn > 4 || step < cn || tw < 1 || th < 1 || tw > iw || th > ih ||
        istride < (int64_t)iw * step || tstride < (int64_t)tw * step) {
        if (err) snprintf(err, 160, "cvmatch: bad match arguments (%dx%d in %dx%d, cn=%d step=%d)", tw, th, iw, ih, cn, step);
        return -1;
    }
    if ((int64_t)tw * th > cvo_stats_cap(cn)) {
        if (err) snprintf(err, 160, "cvmatch: template area %dx%d exceeds the exact-statistics bound for cn=%d", tw, th, cn);
        return -2;
    }
    return 0;
}

int cvo_cross_corr(const uint8_t *img, int64_t istride, int iw, int ih, const uint8_t *tpl,
                   int64_t tstride, int tw, int th, int cn, int step, int threads, float *corr) {
    int rc = check_args(iw, ih, istride, tstride, tw, th, cn, step, NULL);
    if (rc) return rc;
    int rw = iw - tw + 1, rh = ih - th + 1;
    plan_t p;
    plan_make(tw, th, rw, rh, &p);
    plan_tables(&p);
    tset_t set;
    tset_build(tpl, tstride, step, cn, tw, th, rh, th, &p, &set);
    cross_corr(img, istride, step, cn, tw, th, rw, rh, clamp_threads(threads), &p, &set, corr);
    tset_free(&set);
    return 0;
}

/* matchU8, impl.go:1126-1155. */
int cvo_match_u8(const uint8_t *img, int64_t istride, int iw, int ih, const uint8_t *tpl,
                 int64_t tstride, int tw, int th, int cn, int step, int threads, float *result,
                 cvo_result *out, char *err) {
    int rc = check_args(iw, ih, istride, tstride, tw, th, cn, step, err);
    if (rc) return rc;
    threads = clamp_threads(threads);
    int rw = iw - tw + 1, rh = ih - th + 1;
    int64_t tsum[4], varSum;
    cvo_templ_stats(tpl, tstride, tw, th, cn, step, tsum, &varSum);
    if (varSum == 0) {
        if (result) for (size_t i = 0; i < (size_t)rw * rh; i++) result[i] = 1.0f;
        out->min_v = 1.0f; out->min_x = 0; out->min_y = 0;
        out->max_v = 1.0f; out->max_x = 0; out->max_y = 0;
        return 0;
    }
    float *res = result ? result : (float *)malloc(sizeof(float) * (size_t)rw * rh);
    plan_t p;
    plan_make(tw, th, rw, rh, &p);
    plan_tables(&p);
    tset_t set;
    tset_build(tpl, tstride, step, cn, tw, th, rh, th, &p, &set);
    cross_corr(img, istride, step, cn, tw, th, rw, rh, threads, &p, &set, res);
    tset_free(&set);
    normalize_parallel(img, istride, iw, tw, th, cn, step, rw, rh, threads, tsum, varSum, res, res, out);
    if (!result) free(res);
    return 0;
}

/* ---------------------------------------------------- gray and alpha */

void cvo_rgba_to_gray(const uint8_t *pix, int64_t stride, int w, int h, uint8_t *out) {
    for (int y = 0; y < h; y++) {
        const uint8_t *src = pix + (int64_t)y * stride;
        for (int x = 0; x < w; x++) {
            uint32_t r = src[4 * x], g = src[4 * x + 1], b = src[4 * x + 2];
            out[(size_t)y * w + x] = (uint8_t)((4899 * r + 9617 * g + 1868 * b + 8192) >> 14);
        }
    }
}

int cvo_alpha_const(const uint8_t *pix, int64_t stride, int w, int h) {
    uint8_t a = pix[3];
    for (int y = 0; y < h; y++) {
        const uint8_t *row = pix + (int64_t)y * stride;
        for (int x = 0; x < w; x++)
            if (row[4 * x + 3] != a) return 0;
    }
    return 1;
}

/* ---------------------------------------------------------------- fleet */

typedef struct {
    const uint8_t *pix;
    int64_t stride;
    int w, h, step, aConst;
    int64_t tsum[4], varSum;
} member_t;

static void member_init(const cvo_member *m, int step, member_t *o) {
    o->pix = m->pix; o->stride = m->stride; o->w = m->w; o->h = m->h; o->step = step;
    o->aConst = step == 4 ? cvo_alpha_const(m->pix, m->stride, m->w, m->h) : 0;
    /* newMatcher computes the statistics over step channels (matcher.go:75). */
    cvo_templ_stats(m->pix, m->stride, m->w, m->h, step, step, o->tsum, &o->varSum);
}

typedef struct { int pw2, ph2; int *mem; int nm; } cls_t;

static int cls_cmp(const void *a, const void *b) {
    const cls_t *x = (const cls_t *)a, *y = (const cls_t *)b;
    int64_t ax = (int64_t)x->pw2 * x->ph2, ay = (int64_t)y->pw2 * y->ph2;
    if (ax != ay) return ax > ay ? -1 : 1;
    if (x->pw2 != y->pw2) return x->pw2 > y->pw2 ? -1 : 1;
    if (x->ph2 != y->ph2) return x->ph2 > y->ph2 ? -1 : 1;
    return 0;
}

static int int_cmp(const void *a, const void *b) {
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* bucketize, fleet.go:111-171. */
static int bucketize(const member_t *ms, int n, int32_t *btw, int32_t *bth, int32_t *offs, int32_t *mem) {
    cls_t *cls = (cls_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(cls_t));
    int nc = 0;
    for (int i = 0; i < n; i++) {
        if (ms[i].varSum == 0) continue;
        int kw = next_pow2(ms[i].w), kh = next_pow2(ms[i].h);
        int c = -1;
        for (int j = 0; j < nc; j++)
            if (cls[j].pw2 == kw && cls[j].ph2 == kh) { c = j; break; }
        if (c < 0) {
            c = nc++;
            cls[c].pw2 = kw; cls[c].ph2 = kh;
            cls[c].mem = (int *)malloc(sizeof(int) * (size_t)n);
            cls[c].nm = 0;
        }
        cls[c].mem[cls[c].nm++] = i;
    }
    qsort(cls, (size_t)nc, sizeof(cls_t), cls_cmp);
    cls_t *slots = (cls_t *)calloc((size_t)(nc > 0 ? nc : 1), sizeof(cls_t));
    int ns = 0;
    for (int c = 0; c < nc; c++) {
        int placed = 0;
        for (int s = 0; s < ns; s++) {
            if (slots[s].pw2 >= cls[c].pw2 && slots[s].ph2 >= cls[c].ph2) {
                for (int j = 0; j < cls[c].nm; j++) slots[s].mem[slots[s].nm++] = cls[c].mem[j];
                placed = 1;
                break;
            }
        }
        if (!placed) {
            slots[ns].pw2 = cls[c].pw2; slots[ns].ph2 = cls[c].ph2;
            slots[ns].mem = (int *)malloc(sizeof(int) * (size_t)n);
            slots[ns].nm = 0;
            for (int j = 0; j < cls[c].nm; j++) slots[ns].mem[slots[ns].nm++] = cls[c].mem[j];
            ns++;
        }
    }
    int off = 0;
    for (int s = 0; s < ns; s++) {
        qsort(slots[s].mem, (size_t)slots[s].nm, sizeof(int), int_cmp);
        int tw = 0, th = 0;
        offs[s] = off;
        for (int j = 0; j < slots[s].nm; j++) {
            int mi = slots[s].mem[j];
            tw = imax(tw, ms[mi].w);
            th = imax(th, ms[mi].h);
            mem[off++] = mi;
        }
        btw[s] = tw; bth[s] = th;
        free(slots[s].mem);
    }
    offs[ns] = off;
    for (int c = 0; c < nc; c++) free(cls[c].mem);
    free(cls);
    free(slots);
    return ns;
}

int cvo_bucketize(const cvo_member *ms, int n, int step, int32_t *tw, int32_t *th, int32_t *offsets,
                  int32_t *members) {
    member_t *m = (member_t *)malloc(sizeof(member_t) * (size_t)(n > 0 ? n : 1));
    for (int i = 0; i < n; i++) member_init(&ms[i], step, &m[i]);
    int nb = bucketize(m, n, tw, th, offsets, members);
    free(m);
    return nb;
}

/* Phase-2 context: one member's tails against a bucket's frame cache. */
typedef struct {
    const member_t *ms;
    const int32_t *mem;
    int nmem;
    const int *cns;
    const uint8_t *pp;
    int64_t pstride;
    int pw, ph, step, inner;
    const plan_t *p;
    const tset_t *sets;
    const cf *frame;
    const size_t *off;
    int ntx, nty, lastY0;
    cvo_result *out;
    float *const *maps;  /* per member (construction order) score map out, or NULL */
    const uint8_t *want; /* per member (construction order): run its tail; NULL = every member */
    atomic_int next;
    /* phase 1 */
    int btw, bth, rwF, rhF, cnMax, has2;
    const plan_t *p2;
    cf *frame_w;
} fl_ctx;

static void fl_phase1(void *vctx, int w) {
    (void)w;
    fl_ctx *c = (fl_ctx *)vctx;
    const plan_t *p = c->p;
    cf *z = (cf *)malloc(sizeof(cf) * (size_t)p->dftW);
    int ntiles = c->ntx * c->nty;
    for (;;) {
        int t = atomic_fetch_add(&c->next, 1);
        if (t >= ntiles) break;
        int x0 = (t % c->ntx) * p->blockW, y0 = (t / c->ntx) * p->blockH;
        int bwF = imin(p->blockW, c->rwF - x0), bhF = imin(p->blockH, c->rhF - y0);
        const plan_t *bp = (y0 == c->lastY0 && c->has2) ? c->p2 : p;
        size_t sn = (size_t)bp->dftH * bp->hw;
        for (int k = 0; k < c->cnMax; k++)
            block_forward(c->pp + k, c->pstride, c->step, x0, y0, bwF + c->btw - 1, bhF + c->bth - 1, bp,
                          c->frame_w + c->off[t] + (size_t)k * sn, z);
    }
    free(z);
}

static void fl_phase2(void *vctx, int w) {
    (void)w;
    fl_ctx *c = (fl_ctx *)vctx;
    const plan_t *p = c->p;
    size_t specN = (size_t)p->dftH * p->hw;
    cf *spec = (cf *)malloc(sizeof(cf) * specN);
    cf *z = (cf *)malloc(sizeof(cf) * (size_t)p->dftW);
    for (;;) {
        int pos = atomic_fetch_add(&c->next, 1);
        if (pos >= c->nmem) break;
        int mi = c->mem[pos];
        if (c->want && !c->want[mi]) continue;
        const member_t *m = &c->ms[mi];
        int cn = c->cns[mi];
        const tset_t *set = &c->sets[pos];
        int rw = c->pw - m->w + 1, rh = c->ph - m->h + 1;
        float *res = (float *)malloc(sizeof(float) * (size_t)rw * rh);
        int ntiles = c->ntx * c->nty;
        for (int t = 0; t < ntiles; t++) {
            int x0 = (t % c->ntx) * p->blockW, y0 = (t / c->ntx) * p->blockH;
            const plan_t *bp = p;
            const cf *ts = set->spec;
            if (y0 == c->lastY0 && set->has2) { bp = &set->p2; ts = set->spec2; }
            size_t sn = (size_t)bp->dftH * bp->hw;
            int bw = p->blockW, bh = p->blockH;
            if (t % c->ntx == c->ntx - 1) bw = rw - x0;
            if (t / c->ntx == c->nty - 1) bh = rh - y0;
            for (int k = 0; k < cn; k++) {
                memcpy(spec, c->frame + c->off[t] + (size_t)k * sn, sizeof(cf) * sn);
                mul_conj(spec, ts + (size_t)k * sn, sn);
                block_inverse_emit(bp, spec, z, res, rw, x0, y0, bw, bh, k > 0);
            }
        }
        normalize_parallel(c->pp, c->pstride, c->pw, m->w, m->h, cn, c->step, rw, rh, c->inner, m->tsum,
                           m->varSum, res, res, &c->out[mi]);
        if (c->maps && c->maps[mi]) memcpy(c->maps[mi], res, sizeof(float) * (size_t)rw * rh);
        free(res);
    }
    free(spec);
    free(z);
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Fleet.FindAll + buildGeom, fleet.go:176-390; maps (optional, per member
 * in construction order, (pw-w+1) x (ph-h+1) floats each) receive every
 * non-flat member's score map on its bucket's plan.  want (optional, per
 * member in construction order) restricts the member tails (phase 2,
 * fleet.go:265-328) and the member spectra to the members it marks: the
 * buckets, plans and frame spectra stay those of the whole fleet, so a
 * marked member's result is bit-identical to its result in the full
 * FindAll, and unmarked members' results are left untouched.  phase_s
 * (optional) receives the wall seconds of phase 1 (the frame spectra,
 * fleet.go:240-263) and of phase 2, summed over buckets; the member
 * spectra (buildGeom's per-geometry cache, fleet.go:366-375) are in
 * neither. */
int cvo_fleet_find_all_sel(const cvo_member *cms, int n, int step, const uint8_t *pp, int64_t pstride,
                           int pw, int ph, int threads, const uint8_t *want, cvo_result *out,
                           float *const *maps, double *phase_s, char *err) {
    if (phase_s) phase_s[0] = phase_s[1] = 0;
    if (n <= 0) {
        if (err) snprintf(err, 160, "cvmatch: empty fleet");
        return -3;
    }
    threads = clamp_threads(threads);
    member_t *ms = (member_t *)malloc(sizeof(member_t) * (size_t)n);
    for (int i = 0; i < n; i++) member_init(&cms[i], step, &ms[i]);
    for (int i = 0; i < n; i++) {
        if (ms[i].w > pw || ms[i].h > ph) {
            if (err) snprintf(err, 160, "cvmatch: bad match arguments (%dx%d in %dx%d)", ms[i].w, ms[i].h, pw, ph);
            free(ms);
            return -1;
        }
        if (ms[i].varSum == 0) {
            out[i].min_v = 1.0f; out[i].min_x = 0; out[i].min_y = 0;
            out[i].max_v = 1.0f; out[i].max_x = 0; out[i].max_y = 0;
        }
    }
    int32_t *btw = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *bth = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int32_t *offs = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n + 1));
    int32_t *mem = (int32_t *)malloc(sizeof(int32_t) * (size_t)n);
    int nb = bucketize(ms, n, btw, bth, offs, mem);
    int pConst = step == 4 && cvo_alpha_const(pp, pstride, pw, ph);
    int *cns = (int *)calloc((size_t)n, sizeof(int));
    for (int i = 0; i < n; i++) {
        if (ms[i].varSum == 0) continue;
        cns[i] = step == 4 ? ((ms[i].aConst && pConst) ? 3 : 4) : 1;
    }
    for (int b = 0; b < nb; b++) {
        const int32_t *bm = mem + offs[b];
        int nm = offs[b + 1] - offs[b];
        int rwF = pw - btw[b] + 1, rhF = ph - bth[b] + 1;
        plan_t p;
        plan_make(btw[b], bth[b], rwF, rhF, &p);
        plan_tables(&p);
        plan_t p2 = p;
        int dh2 = shrink_dh(&p, rhF, bth[b]);
        if (dh2 > 0) {
            p2.dftH = dh2;
            p2.tH = tables(dh2);
        }
        tset_t *sets = (tset_t *)calloc((size_t)nm, sizeof(tset_t));
        int cnMax = 0;
        for (int j = 0; j < nm; j++) {
            const member_t *m = &ms[bm[j]];
            int cn = cns[bm[j]];
            cnMax = imax(cnMax, cn);
            if (!want || want[bm[j]]) tset_build(m->pix, m->stride, step, cn, m->w, m->h, rhF, bth[b], &p, &sets[j]);
        }
        int ntx = (rwF + p.blockW - 1) / p.blockW;
        int nty = (rhF + p.blockH - 1) / p.blockH;
        int ntiles = ntx * nty;
        int lastY0 = ((rhF - 1) / p.blockH) * p.blockH;
        size_t *off = (size_t *)malloc(sizeof(size_t) * (size_t)(ntiles + 1));
        off[0] = 0;
        for (int t = 0; t < ntiles; t++) {
            int y0 = (t / ntx) * p.blockH;
            const plan_t *bp = (y0 == lastY0 && dh2 > 0) ? &p2 : &p;
            off[t + 1] = off[t] + (size_t)cnMax * bp->dftH * bp->hw;
        }
        cf *frame = (cf *)malloc(sizeof(cf) * (off[ntiles] > 0 ? off[ntiles] : 1));
        fl_ctx c;
        memset(&c, 0, sizeof c);
        c.ms = ms; c.mem = bm; c.nmem = nm; c.cns = cns; c.pp = pp; c.pstride = pstride;
        c.pw = pw; c.ph = ph; c.step = step; c.p = &p; c.sets = sets; c.frame = frame; c.off = off;
        c.ntx = ntx; c.nty = nty; c.lastY0 = lastY0; c.out = out;
        c.btw = btw[b]; c.bth = bth[b]; c.rwF = rwF; c.rhF = rhF; c.cnMax = cnMax;
        c.has2 = dh2 > 0; c.p2 = &p2; c.frame_w = frame; c.maps = maps; c.want = want;
        atomic_init(&c.next, 0);
        double t0 = now_s();
        run_parallel(imin(threads, ntiles), fl_phase1, &c);
        double t1 = now_s();
        int outer = imin(threads, nm);
        c.inner = imax(threads / outer, 1);
        atomic_store(&c.next, 0);
        run_parallel(outer, fl_phase2, &c);
        if (phase_s) {
            phase_s[0] += t1 - t0;
            phase_s[1] += now_s() - t1;
        }
        for (int j = 0; j < nm; j++)
            if (!want || want[bm[j]]) tset_free(&sets[j]);
        free(sets);
        free(off);
        free(frame);
    }
    free(cns);
    free(btw); free(bth); free(offs); free(mem);
    free(ms);
    return 0;
}

int cvo_fleet_find_all_maps(const cvo_member *cms, int n, int step, const uint8_t *pp, int64_t pstride,
                            int pw, int ph, int threads, cvo_result *out, float *const *maps, char *err) {
    return cvo_fleet_find_all_sel(cms, n, step, pp, pstride, pw, ph, threads, NULL, out, maps, NULL, err);
}

int cvo_fleet_find_all(const cvo_member *cms, int n, int step, const uint8_t *pp, int64_t pstride,
                       int pw, int ph, int threads, cvo_result *out, char *err) {
    return cvo_fleet_find_all_maps(cms, n, step, pp, pstride, pw, ph, threads, out, NULL, err);
}

/* --------------------------------------------------------- FP64 oracle */

typedef struct {
    const uint8_t *img;
    int64_t istride;
    const uint8_t *tpl;
    int64_t tstride;
    int tw, th, cn, step, rw, rh, nthr;
    double templNorm, invArea;
    const double *mean;
    double *out;
} rf_ctx;

static void rf_worker(void *vctx, int w) {
    rf_ctx *c = (rf_ctx *)vctx;
    for (int y = w; y < c->rh; y += c->nthr) {
        for (int x = 0; x < c->rw; x++) {
            double corr = 0, wsum[4] = {0, 0, 0, 0}, wsum2 = 0;
            for (int dy = 0; dy < c->th; dy++) {
                const uint8_t *ir = c->img + (int64_t)(y + dy) * c->istride + (int64_t)x * c->step;
                const uint8_t *tr = c->tpl + (int64_t)dy * c->tstride;
                for (int dx = 0; dx < c->tw; dx++)
                    for (int k = 0; k < c->cn; k++) {
                        double iv = ir[dx * c->step + k], tv = tr[dx * c->step + k];
                        corr += iv * tv;
                        wsum[k] += iv;
                        wsum2 += iv * iv;
                    }
            }
            double num = corr, wm2 = 0;
            for (int k = 0; k < c->cn; k++) {
                wm2 += wsum[k] * wsum[k];
                num -= wsum[k] * c->mean[k];
            }
            wm2 *= c->invArea;
            double diff2 = wsum2 - wm2;
            if (diff2 < 0) diff2 = 0;
            double lim = 1.1920929e-06 * wsum2; /* Go folds the constant 10*fltEps exactly */
            if (lim > 0.5) lim = 0.5;
            double den = 0;
            if (diff2 > lim) den = sqrt(diff2) * c->templNorm;
            if (fabs(num) < den) num /= den;
            else if (fabs(num) < den * 1.125) num = copysign(1.0, num);
            else num = 0;
            c->out[(size_t)y * c->rw + x] = num;
        }
    }
}

/* refMatch, cvmatch_test.go:13-81. */
void cvo_ref_match_f64(const uint8_t *img, int64_t istride, int iw, int ih, const uint8_t *tpl,
                       int64_t tstride, int tw, int th, int cn, int step, int threads, double *out) {
    double area = (double)(tw * th), invArea = 1 / area;
    double mean[4] = {0, 0, 0, 0}, templNorm = 0;
    for (int k = 0; k < cn; k++) {
        double s = 0, s2 = 0;
        for (int y = 0; y < th; y++)
            for (int x = 0; x < tw; x++) {
                double v = tpl[(int64_t)y * tstride + x * step + k];
                s += v;
                s2 += v * v;
            }
        mean[k] = s * invArea;
        templNorm += s2 * invArea - mean[k] * mean[k];
    }
    int rw = iw - tw + 1, rh = ih - th + 1;
    if (templNorm < 2.220446049250313e-16) {
        for (size_t i = 0; i < (size_t)rw * rh; i++) out[i] = 1;
        return;
    }
    templNorm = sqrt(templNorm * area);
    if (threads < 1) threads = 1;
    if (threads > 64) threads = 64;
    rf_ctx c = {img, istride, tpl, tstride, tw, th, cn, step, rw, rh, threads, templNorm, invArea, mean, out};
    run_parallel(threads, rf_worker, &c);
}
