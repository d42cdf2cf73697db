/*
 * cvm_oracle.h -- CPU restatement of cvmatch's TM_CCOEFF_NORMED path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product is compared against; it is never linked into, loaded by, or
 * called from the product library (cvmatch_gb300/csrc).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may use it.
 *
 * It restates the reference's scalar Go path op for op (float32 single
 * rounding, no fused multiply-add, the same deterministic twiddles), so
 * on the same inputs it reproduces the reference's output bits.  The
 * pins that prove this (golden hash of case 110, the 15 plan pins, the
 * statistics caps, the bucketing pins) live in tests/test_oracle_pins.py.
 */
#ifndef CVM_ORACLE_H
#define CVM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    float min_v;
    int32_t min_x, min_y;
    float max_v;
    int32_t max_x, max_y;
} cvo_result;

typedef struct {
    int32_t dft_w, dft_h, hw, block_w, block_h;
    int64_t cost;
} cvo_plan;

/* newGoPlan (impl.go:246-295). */
void cvo_plan_make(int tw, int th, int rw, int rh, cvo_plan *out);
/* shrinkDH (impl.go:573-582): 0 when the last band keeps dftH. */
int cvo_shrink_dh(const cvo_plan *p, int rh, int th);
/* statsCap (impl.go:1122-1124). */
int64_t cvo_stats_cap(int cn);

/* sincospiFrac (impl.go:98-133). */
void cvo_sincospi(int j, int half, float *c, float *s);
/* makeTriTwiddles (radix4.go:45-73); returns the number of complex
 * entries written to tri (interleaved re,im floats), tri may be NULL. */
int cvo_tri_twiddles(int n, float *tri);
/* fftR4 (radix4.go:91-149), in place on n interleaved complex floats. */
void cvo_fft_r4(float *a, int n, int inverse);
/* colsR4Go (radix4cols.go:111-125) on a row-major [n x width] slab;
 * use_rmap selects the bit-reversed row map of the inverse path. */
void cvo_cols_r4(float *d, int n, int width, int inverse, int use_rmap);

/* rgbToGray (cvmatch.go:222-240); out is w*h bytes. */
void cvo_rgba_to_gray(const uint8_t *pix, int64_t stride, int w, int h, uint8_t *out);
/* alphaConst (cvmatch.go:146-168). */
int cvo_alpha_const(const uint8_t *pix, int64_t stride, int w, int h);

/* templStats (impl.go:1063-1079). */
void cvo_templ_stats(const uint8_t *tpl, int64_t tstride, int tw, int th, int cn,
                     int step, int64_t tsum[4], int64_t *var_sum);

/* matchU8 (impl.go:1126-1155).  result may be NULL.  Returns 0, or a
 * negative code with the reference's panic text in err (>=160 bytes). */
int cvo_match_u8(const uint8_t *img, int64_t istride, int iw, int ih,
                 const uint8_t *tpl, int64_t tstride, int tw, int th, int cn,
                 int step, int threads, float *result, cvo_result *out, char *err);

/* Raw cross-correlation only (crossCorrGo, impl.go:616-693), the map the
 * normalization consumes; used to isolate the stages in tests. */
int cvo_cross_corr(const uint8_t *img, int64_t istride, int iw, int ih,
                   const uint8_t *tpl, int64_t tstride, int tw, int th, int cn,
                   int step, int threads, float *corr);

/* Normalization + scan only (normalizeParallelGo, impl.go:1081-1114) over
 * a given raw correlation map; result may alias corr. */
void cvo_normalize(const uint8_t *img, int64_t istride, int iw, int ih, int tw, int th,
                   int cn, int step, const int64_t tsum[4], int64_t var_sum,
                   int threads, const float *corr, float *result, cvo_result *out);

/* Fleet (fleet.go).  Members are given as raw template pixels with the
 * Matcher's step (4 colour, 1 gray); all members share one step. */
typedef struct {
    const uint8_t *pix;
    int64_t stride;
    int32_t w, h;
} cvo_member;

/* bucketize (fleet.go:111-171).  Writes, per bucket b, its tw/th and the
 * member list into members[offsets[b]..offsets[b+1]).  Returns the bucket
 * count.  Arrays must hold n entries (offsets n+1). */
int cvo_bucketize(const cvo_member *ms, int n, int step, int32_t *tw, int32_t *th,
                  int32_t *offsets, int32_t *members);

/* Fleet.FindAll (fleet.go:176-332) for a fleet built from ms. */
int cvo_fleet_find_all(const cvo_member *ms, int n, int step, const uint8_t *parent,
                       int64_t pstride, int pw, int ph, int threads, cvo_result *out,
                       char *err);
int cvo_fleet_find_all_maps(const cvo_member *cms, int n, int step, const uint8_t *pp, int64_t pstride,
                            int pw, int ph, int threads, cvo_result *out, float *const *maps, char *err);
/* The same restricted to the members want marks (NULL: all), on the whole
 * fleet's buckets and plans (marked members' results are bit-identical to
 * the full FindAll's); phase_s (nullable) gets the seconds of phase 1 and
 * phase 2. */
int cvo_fleet_find_all_sel(const cvo_member *cms, int n, int step, const uint8_t *pp, int64_t pstride,
                           int pw, int ph, int threads, const uint8_t *want, cvo_result *out,
                           float *const *maps, double *phase_s, char *err);

/* Brute-force FP64 TM_CCOEFF_NORMED from the definition
 * (cvmatch_test.go:13-81); out has rw*rh doubles. */
void cvo_ref_match_f64(const uint8_t *img, int64_t istride, int iw, int ih,
                       const uint8_t *tpl, int64_t tstride, int tw, int th, int cn,
                       int step, int threads, double *out);

#ifdef __cplusplus
}
#endif
#endif
