/*
 * cvmatch_gpu.h -- C ABI of the GB300 (sm_103a) TM_CCOEFF_NORMED engine.
 *
 * This is the boundary a cgo shim binds in place of cvmatch's Go core
 * (L3-L1: impl.go, radix4.go, radix4cols.go, internal/simd).  The Go
 * package keeps its public API and its image adaptation (toRGBA/toGray,
 * cvmatch.go:186-217) and passes raw (pointer, stride, width, height)
 * views across; nothing here takes Go or torch types.
 *
 * Conventions
 *   - Every function returns CVM_OK (0) or a nonzero CVM_ERR_* code; the
 *     message of the last failure on the calling thread is available from
 *     cvm_last_error().  Argument errors carry the reference's exact panic
 *     text, so the Go shim can re-panic with the identical string.
 *   - Host-buffer entry points copy their inputs to the device inside the
 *     call and return after the results are back on the host; the caller
 *     keeps ownership of every buffer and may reuse it after return (cgo's
 *     pointer rules forbid retaining Go memory, and nothing is retained).
 *   - RGBA images are interleaved 4 bytes per pixel; gray images 1 byte.
 *     Strides are in bytes and may exceed width*bytes-per-pixel
 *     (sub-images).
 *   - All entry points are safe for concurrent use from several threads.
 *     Handles serialise their own lazy geometry builds.
 *   - One device per process: the library binds to the CUDA device that is
 *     current on the calling thread at its first call (its memory pool,
 *     tables, streams and every Matcher/Fleet cache live there); a later
 *     call made with a different device current returns
 *     CVM_ERR_UNSUPPORTED before queueing anything.  (The fixed-scratch
 *     entry point keeps its own per-device set-up.)
 *   - The computation is the reference's op sequence: scores are
 *     bit-identical to cvmatch's Go path on the same inputs.
 */
#ifndef CVMATCH_GPU_H
#define CVMATCH_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Match's six-tuple; the reference's Fleet Result (fleet.go:13-18). */
typedef struct cvm_result {
    float min_v;
    int32_t min_x, min_y;
    float max_v;
    int32_t max_x, max_y;
} cvm_result;

typedef struct cvm_matcher cvm_matcher;
typedef struct cvm_fleet cvm_fleet;

enum {
    CVM_OK = 0,
    CVM_ERR_ARGS = 1,        /* "cvmatch: bad match arguments (...)"  impl.go:1127-1130, matcher.go:97-99, fleet.go:192-194 */
    CVM_ERR_STATS_CAP = 2,   /* "cvmatch: template area ... exceeds the exact-statistics bound ..." impl.go:1131-1133, matcher.go:67-69 */
    CVM_ERR_EMPTY_FLEET = 3, /* "cvmatch: empty fleet"  fleet.go:86-88 */
    CVM_ERR_MIXED_FLEET = 4, /* "cvmatch: fleet mixes color and gray matchers"  fleet.go:93-97 */
    CVM_ERR_NIL_IMAGE = 5,   /* "cvmatch: nil image"  cvmatch.go:170-173 */
    CVM_ERR_EMPTY_IMAGE = 6, /* "cvmatch: empty image"  cvmatch.go:174-177 */
    CVM_ERR_CUDA = 10,       /* a CUDA runtime call failed (message names it) */
    CVM_ERR_UNSUPPORTED = 11,/* a transform size beyond the library's limits */
    CVM_ERR_NO_DEVICE = 12   /* no sm_103 device / the library was not built for it */
};

/* Copies the calling thread's last error message (NUL-terminated,
 * truncated to len) and returns its full length. */
size_t cvm_last_error(char *buf, size_t len);

/* ------------------------------------------------- one-shot entry points */

/* Match (cvmatch.go:75-94): parent and sub are RGBA; the alpha channel is
 * skipped exactly when both alpha planes are constant (cvmatch.go:82-85). */
int cvm_match(const uint8_t *parent, int64_t pstride, int pw, int ph,
              const uint8_t *sub, int64_t sstride, int sw, int sh, cvm_result *out);

/* MatchMap (cvmatch.go:100-117): as cvm_match, and fills map with the
 * (pw-sw+1) x (ph-sh+1) row-major float32 response. */
int cvm_match_map(const uint8_t *parent, int64_t pstride, int pw, int ph,
                  const uint8_t *sub, int64_t sstride, int sw, int sh, float *map);

/* MatchGray (cvmatch.go:128-139) on 8-bit gray planes (the zero-copy
 * *image.Gray / *image.YCbCr Y-plane case of toGray, cvmatch.go:205-208). */
int cvm_match_gray(const uint8_t *parent, int64_t pstride, int pw, int ph,
                   const uint8_t *sub, int64_t sstride, int sw, int sh, cvm_result *out);

/* MatchGray on RGBA/NRGBA inputs: both images are converted on the device
 * with rgbToGray's fixed-point weights (cvmatch.go:209-212, 222-240). */
int cvm_match_gray_rgba(const uint8_t *parent, int64_t pstride, int pw, int ph,
                        const uint8_t *sub, int64_t sstride, int sw, int sh, cvm_result *out);

/* matchU8 (impl.go:1126-1155): the generic core every entry point funnels
 * into.  cn channels of step-byte pixels; map may be NULL. */
int cvm_match_u8(const uint8_t *img, int64_t istride, int iw, int ih,
                 const uint8_t *tpl, int64_t tstride, int tw, int th, int cn, int step,
                 float *map, cvm_result *out);

/* Device-resident matchU8: img/tpl/map/out are device pointers, the work
 * is queued on stream (a cudaStream_t, NULL = legacy default stream) and
 * the call returns without synchronising. */
int cvm_match_u8_device(const uint8_t *d_img, int64_t istride, int iw, int ih,
                        const uint8_t *d_tpl, int64_t tstride, int tw, int th, int cn, int step,
                        float *d_map, cvm_result *d_out, void *stream);

/* Device-resident Match: colour semantics with the alpha decision made on
 * the device (no host round trip). */
int cvm_match_device(const uint8_t *d_parent, int64_t pstride, int pw, int ph,
                     const uint8_t *d_sub, int64_t sstride, int sw, int sh,
                     float *d_map, cvm_result *d_out, void *stream);

/* matchU8 on device buffers without allocating device memory.  This entry
 * point has no counterpart in the reference.  It is for callers that must
 * not allocate: code running inside a memory budget another allocator owns
 * (a framework's caching pool, a runtime that reserves the device at
 * start-up) or loops where a driver allocation's latency is unacceptable.
 * The workspace is one fixed 64 MiB device array inside the library, held
 * by every GPU that loads it until the process exits; a match whose
 * workspace does not fit (roughly: colour frames above ~2 Mpx, gray frames
 * above ~6 Mpx) returns CVM_ERR_UNSUPPORTED.  The caller passes inputs and
 * outputs as for cvm_match_u8_device.  The first call on a device sets the
 * array up (synchronous copies of the twiddle tables); make that first call
 * before any stream capture.  All calls share the array: calls whose work
 * overlaps on the GPU race, so serialise them.  It always computes the
 * exact form (the reference's float32 op sequence, bit-identical to
 * cvm_match_u8_device in CVM_FORM_EXACT), whatever cvm_set_form selects,
 * and refuses templates so wide that its normalisation would need more
 * shared memory per block than the device has (CVM_ERR_UNSUPPORTED). */
int cvm_match_u8_device_noalloc(const uint8_t *d_img, int64_t istride, int iw, int ih,
                                const uint8_t *d_tpl, int64_t tstride, int tw, int th, int cn, int step,
                                float *d_map, cvm_result *d_out, void *stream);

/* ----------------------------------------------------- image primitives */

/* rgbToGray (cvmatch.go:222-240): out is w*h packed gray bytes. */
int cvm_rgba_to_gray(const uint8_t *pix, int64_t stride, int w, int h, uint8_t *out);

/* rgbToGray on device buffers: d_out (row stride ostride bytes) receives
 * the gray plane of the RGBA image d_pix; queued on stream without
 * synchronising.  MatchGray converts both of its inputs on every call
 * (cvmatch.go:128-139, toGray cvmatch.go:201-217); a device-resident caller
 * converts with this and then calls cvm_match_u8_device with cn = step = 1. */
int cvm_rgba_to_gray_device(const uint8_t *d_pix, int64_t stride, int w, int h, uint8_t *d_out, int64_t ostride,
                            void *stream);

/* alphaConst (cvmatch.go:146-168): *out = 1 when every alpha byte equals
 * the first pixel's. */
int cvm_alpha_const(const uint8_t *pix, int64_t stride, int w, int h, int *out);

/* ------------------------------------------------------------- Matcher */

/* newMatcher (matcher.go:45-76): step 4 = NewMatcher (RGBA, Match
 * semantics), step 1 = NewGrayMatcher (gray plane, MatchGray semantics).
 * The pixels are copied; the template statistics are computed here. */
int cvm_matcher_new(const uint8_t *pix, int64_t stride, int w, int h, int step, cvm_matcher **out);

/* Matcher.Find (matcher.go:83-130): bit-identical to Match / MatchGray. */
int cvm_matcher_find(cvm_matcher *m, const uint8_t *parent, int64_t pstride, int pw, int ph,
                     cvm_result *out);

/* Device-resident Find: d_parent and d_out are device pointers; queued on
 * stream without synchronising. */
int cvm_matcher_find_device(cvm_matcher *m, const uint8_t *d_parent, int64_t pstride, int pw, int ph,
                            cvm_result *d_out, void *stream);

void cvm_matcher_free(cvm_matcher *m);

/* ---------------------------------------------------- every occurrence */

/* The MatchMap recipe for every occurrence (cvmatch_test.go:324-381,
 * README.md:82-90) on the device: (x, y) is an occurrence when its score is
 * not below thresh and no score within dx in [-rx, rx], dy in [-ry, ry]
 * (clipped to the map) is strictly greater.  *count receives the number of
 * occurrences, xy the first max_peaks of them in raster order as (x, y)
 * pairs.  The map never leaves the device.  No reference counterpart as a
 * function: the reference leaves the recipe to its callers. */
int cvm_match_map_peaks(const uint8_t *parent, int64_t pstride, int pw, int ph, const uint8_t *sub, int64_t sstride,
                        int sw, int sh, float thresh, int rx, int ry, int32_t *xy, int max_peaks, int32_t *count);
/* The same on matchU8's raw views (impl.go:1126-1155). */
int cvm_match_u8_peaks(const uint8_t *img, int64_t istride, int iw, int ih, const uint8_t *tpl, int64_t tstride,
                       int tw, int th, int cn, int step, float thresh, int rx, int ry, int32_t *xy, int max_peaks,
                       int32_t *count);
/* The recipe on a device-resident w x h map (from cvm_match_u8_device or
 * cvm_match_device); d_xy/d_count are device pointers; queued on stream. */
int cvm_peaks_device(const float *d_map, int w, int h, float thresh, int rx, int ry, int32_t *d_xy, int max_peaks,
                     int32_t *d_count, void *stream);

/* --------------------------------------------------------------- Fleet */

/* NewFleet (fleet.go:85-101): the member list is copied; the matchers must
 * outlive the fleet.  All members share one mode. */
int cvm_fleet_new(cvm_matcher *const *ms, int n, cvm_fleet **out);

/* Fleet.FindAll (fleet.go:176-332): out receives n results in
 * construction order. */
int cvm_fleet_find_all(cvm_fleet *f, const uint8_t *parent, int64_t pstride, int pw, int ph,
                       cvm_result *out);

/* Device-resident FindAll: d_parent/d_out are device pointers (d_out holds
 * n results); queued on stream without synchronising. */
int cvm_fleet_find_all_device(cvm_fleet *f, const uint8_t *d_parent, int64_t pstride, int pw, int ph,
                              cvm_result *d_out, void *stream);

void cvm_fleet_free(cvm_fleet *f);

/* Region of interest of one member (construction order), x, y, w, h in
 * frame pixels; w or h <= 0 clears it.  The member's result is the
 * first-occurrence extrema of its FindAll score map over the positions
 * whose window lies inside the ROI, in frame coordinates; tiles and rows
 * outside it are skipped.  An ROI that cannot hold the template gives
 * min_v = max_v = NaN and positions -1.  (The reference keeps per-ROI
 * crop fleets instead, examples/windowrules/engine.go:276-343; per-member
 * ROIs on the shared frame spectra are its parked item, CLAUDE.md:463-475.)
 * Not to be called while a FindAll on the same fleet runs. */
int cvm_fleet_set_roi(cvm_fleet *f, int member, int x, int y, int w, int h);

/* Arithmetic of a fleet's member tails.  CVM_FORM_EXACT (the default) is
 * the reference's float32 pipeline op for op: every score equals
 * Fleet.FindAll's bit for bit (fleet.go:176-332, impl.go:301-464,
 * 825-849).  CVM_FORM_FAST gives up that bit identity for throughput and
 * conditioning: templates enter as their zero-mean form area*T - sum(T)
 * (exact integers), the frame as I - 128, so the correlation is the
 * TM_CCOEFF_NORMED numerator itself (no float32 cancellation against
 * sum(I)*sum(T)/area); the channels of a member are summed in the
 * frequency domain, so each member tile takes one inverse transform
 * instead of one per channel; the window statistics and the score
 * ladder stay those of normOne.  Scores then differ from the reference's
 * by rounding only (bounded against the FP64 definition in the tests).
 * Changing the form drops the fleet's cached spectra; not to be called
 * while a FindAll on the same fleet runs.  A bucket (or one-shot match)
 * whose plan needs transforms above 4096 points -- templates over ~4000
 * pixels on a side -- runs the exact form's kernels instead, whatever the
 * form: its scores are then the reference's bits. */
enum { CVM_FORM_EXACT = 0, CVM_FORM_FAST = 1, CVM_FORM_MIXED = 2 };
int cvm_fleet_set_form(cvm_fleet *f, int form);

/* The same choice for one-shot matches (cvm_match, cvm_match_map,
 * cvm_match_gray*, cvm_match_u8*, cvm_match_device and the peaks entry
 * points) and Matcher.Find, process-wide, read at the start of each call
 * (a Matcher rebuilds its cached spectra when the form changed).  In the
 * fast form each tile's channels are transformed forward, their
 * conj-products summed, and one inverse taken; the score map is the fast
 * form's.  The reference has no such switch (its Threads variable,
 * cvmatch.go:42, is the nearest process-wide knob); the default stays
 * CVM_FORM_EXACT.  cvm_match_u8_device_noalloc always computes the exact
 * form. */
int cvm_set_form(int form);
int cvm_get_form(void);

/* CVM_FORM_MIXED (fleets and one-shot matches alike) is the fast form with
 * its 1024-point inverse row transforms -- the inverse DFT of inverseRowPair
 * (impl.go:394-444) -- run on the tensor cores: two 32-point DFT stages as
 * tcgen05 kind::f16 matrix products on operands scaled per transform by a
 * power of two and split into FP16 hi + lo halves (three products, FP32
 * accumulation), the twiddles between them in FP32.  Other transform
 * widths run the fast form unchanged.  Scores differ from the fast form's
 * by rounding only. */

/* The tile-plan autotuner of the fast and mixed forms (on by default; the
 * exact form always runs newGoPlan's plan, impl.go:246-295, since its bits
 * depend on it).  The first fast-form one-shot match or Matcher.Find of a
 * shape (frame size, template size, channel mode, form) times up to four
 * power-of-two tile plans on its own inputs, each from a cold L2 (a
 * transient device buffer of twice the L2's size is cleared before each
 * timed run) -- newGoPlan's choice and the best of a GPU cost proxy -- and
 * keeps the fastest if it beats newGoPlan's
 * by more than 3 %; every later call of that shape in the process runs the
 * cached plan (so results repeat exactly).  A fleet's first fast-form
 * FindAll of a frame size does the same per bucket of four or more members
 * (buildGeom's plan, fleet.go:356-365, against the candidates), timing
 * trial fleets of k and 2k of the bucket's own members so that the cost is
 * shared + members x per-member.  Calls made while their stream is being
 * captured do not tune.  cvm_set_autotune returns the previous setting.
 * No reference counterpart (the reference always plans with newGoPlan). */
int cvm_set_autotune(int on);
/* The tuned shapes as a JSON array (frame, template, mode, cn, step, form,
 * the chosen plan and each candidate's measured ms; fleet buckets with
 * "fleet": true, the bucket maxima, members and each candidate's per-member
 * and shared ms); returns the full length, writes at most len - 1
 * characters and a terminating NUL. */
size_t cvm_autotune_report(char *buf, size_t len);

/* Checks the tensor-core DFT path on this device: four inverse 1024-point
 * DFTs through the kernel's own stages against a double-precision DFT on
 * the host.  *dft_err and *gemm_err receive the largest errors relative to
 * each line's norm (of the whole DFT, and of the first GEMM stage alone).
 * Diagnostic; no reference counterpart. */
int cvm_tc_selftest(double *dft_err, double *gemm_err);

/* Sticky device-side failure flags since the last call (then cleared):
 * *tc_timeouts = 1 when a kernel gave up waiting for its asynchronous
 * hardware -- the tensor-core DFT for its matrix products, the forward
 * rows for their TMA frame copies -- and its results are invalid.  Waits
 * are bounded, so such a failure returns instead of hanging.  No reference
 * counterpart. */
int cvm_device_status(int *tc_timeouts);

/* ------------------------------------------------------- frame streams */

/* A stream of RGBA frames of one size matched against a colour fleet and,
 * optionally, a gray fleet on each frame's gray conversion (rgbToGray,
 * cvmatch.go:222-240) -- the loop a caller would write around
 * Fleet.FindAll (fleet.go:176-332) for a video feed; no reference
 * counterpart as an object.  The per-frame pipeline (frame upload, both
 * FindAlls, the gray conversion, result read-back) is captured once as a
 * CUDA graph per frame slot and replayed; two slots let one frame's upload
 * overlap the previous frame's matching.  Results are identical to calling
 * cvm_fleet_find_all per frame.  The fleets must outlive the stream. */
typedef struct cvm_stream cvm_stream;
int cvm_stream_new(cvm_fleet *color, cvm_fleet *gray_or_null, int pw, int ph, cvm_stream **out);
/* Queue one frame (pw x ph RGBA, row stride in bytes); the pixels are
 * copied before the call returns.  With both slots in flight it first
 * waits for the oldest frame. */
int cvm_stream_push(cvm_stream *s, const uint8_t *rgba, int64_t stride);
/* Results of the oldest queued frame (waits for it): color_out receives the
 * colour fleet's n results, gray_out the gray fleet's (may be null without
 * one); device_ms (nullable) the frame's upload-to-results time. */
int cvm_stream_pull(cvm_stream *s, cvm_result *color_out, cvm_result *gray_out, double *device_ms);
/* 1 when the per-frame pipeline runs as a CUDA graph, 0 when it is issued
 * launch by launch (capture unavailable); kernels per frame in *launches. */
int cvm_stream_info(cvm_stream *s, int *graphed, int *launches);
void cvm_stream_free(cvm_stream *s);

/* ------------------------------------------------------------- support */

/* The tile geometry the library plans for a tw x th template over a
 * rw x rh result (newGoPlan, impl.go:246-295, and the shrunk last band of
 * shrinkDH, impl.go:573-582): out = {dftW, dftH, blockW, blockH, dh2,
 * tiles}, dh2 = 0 when the last band keeps dftH.  Host-only; no device. */
int cvm_plan(int tw, int th, int rw, int rh, int32_t out[6]);

/* A fleet's buckets (bucketize, fleet.go:111-171) and each bucket's plan on
 * a pw x ph frame (buildGeom, fleet.go:356-365): returns the bucket count
 * (negative on error) and, for the first cap buckets, 9 ints each: {tw,
 * th, dftW, dftH, blockW, blockH, dh2, tiles, members} -- newGoPlan's
 * plan (the exact form's; the fast forms may run a tuned one, listed by
 * cvm_autotune_report).  Flat members are in no bucket.  Host-only; no
 * device. */
int cvm_fleet_buckets(const cvm_fleet *f, int pw, int ph, int32_t *out, int cap);
/* At most `members` member tails per wave of a FindAll (0, the default:
 * as few waves as a 4 GB workspace allows, of equal size).  Each wave's tails write their
 * column-pass spectra (~25 MB per member on a 2560x1440 frame) before the
 * row pass reads them back: small waves bound the workspace and keep those
 * spectra in L2, large waves need fewer launches.  Results do not depend
 * on it.  Not to be called while a FindAll on the same fleet runs. */
int cvm_fleet_set_wave(cvm_fleet *f, int members);
/* Overlapped waves (on, the default): a fast-form FindAll with more than
 * one wave of member tails runs the inverse rows of wave k on a second
 * stream beside the window statistics and column pass of wave k + 1 (the
 * waves alternate between two workspaces); off, and in the exact and mixed
 * forms (slower overlapped), every wave's launches run in sequence on the
 * caller's stream.  Results do not depend on it.  No reference
 * counterpart.  Not to be called while a FindAll on the same fleet runs. */
int cvm_fleet_set_overlap(cvm_fleet *f, int on);

/* Where a fleet's window statistics are formed (no counterpart in the
 * reference, which computes them in normalizeBandGo, impl.go:708-805).
 * CVM_STATS_KERNEL (the default): the statistics kernel writes each
 * window's den, which the inverse-rows epilogue reads back.
 * CVM_STATS_EPILOGUE: fast-form buckets without regions of interest whose
 * every member satisfies area * cn * 16256 < 2^32 (colour members up to
 * 66,052 px, gray up to 264,208 px) form each window's den inside the
 * inverse-rows epilogue from the frame's summed-area table, with no
 * statistics launch and no den written or read; other buckets, and every
 * exact- or mixed-form bucket, still run the statistics kernel.  Results
 * are the same bits either way.  The epilogue form measured slower on a
 * GB300 (256 RGBA templates on a 2560x1440 frame: 10.3 against 9.5 ms per
 * FindAll), hence not the default.  Not to be called while a FindAll on
 * the same fleet runs. */
#define CVM_STATS_KERNEL 0
#define CVM_STATS_EPILOGUE 1
int cvm_fleet_set_stats(cvm_fleet *f, int mode);

/* Bucket b's members (construction-order indices, ascending): returns
 * their count (negative on error) and writes the first cap of them. */
int cvm_fleet_bucket_members(const cvm_fleet *f, int b, int32_t *out, int cap);

/* Page-locked host memory for frames the caller wants copied at full
 * host-to-device bandwidth (plain pageable memory also works). */
void *cvm_host_alloc(size_t bytes);
void cvm_host_free(void *p);

/* Number of this library's kernels launched since load (a counter the
 * benchmark reads to report launches per step). */
uint64_t cvm_launch_count(void);

/* Per-kernel timing for profiling runs: while enabled, every kernel launch
 * is bracketed by CUDA events recorded on its own stream (off by default;
 * enabling clears earlier totals).  cvm_profile_read(i, ...) returns 0 and
 * the i-th kernel's name, total milliseconds and launch count, or nonzero
 * past the last kernel; it waits for the recorded events. */
void cvm_profile_enable(int on);
int cvm_profile_read(int i, char *name, size_t len, double *ms_total, uint64_t *launches);
/* The i-th profiled launch in completion-collection order: its kernel name
 * and its start and end in milliseconds after the first profiled launch's
 * start (a timeline across streams); nonzero past the last launch.
 * Profiling aid with no reference counterpart. */
int cvm_profile_span(int i, char *name, size_t len, double *t0_ms, double *t1_ms);

/* Library version string. */
const char *cvm_version(void);

#ifdef __cplusplus
}
#endif
#endif
