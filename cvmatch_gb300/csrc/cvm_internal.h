// cvm_internal.h -- structures shared by the host orchestration
// (cvm_api.cpp, cvm_plan.cpp) and the sm_103a kernels (cvm_kernels.cu).
//
// Data layout in HBM (one frame, one bucket/plan class):
//   frame        u8, device copy of the caller's image, pitch = stride
//   window sums  per image row, the horizontal window sums of every
//                channel and of the squared pixels (u32, modular: every
//                window sum is < 2^32), interleaved per x; a fleet keeps
//                one set of exclusive row prefixes instead
//   lanes        per result (t, den): the correlation-free part of normOne
//   spectra      per tile t and channel k a dftH x hwp complex64 slab
//                (hwp = dftW/2+1 rounded up to 16): the forward rows
//                kernel writes logical spectrum row L at slot brev(L),
//                the column kernel leaves spatial row y at slot brev(y)
//                (the reference's storage relabelling, radix4cols.go:12-24)
//   partials     one (min,max,index) record per inverse-rows CTA
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "cvmatch_gpu.h"

namespace cvm {

// newGoPlan's result (impl.go:227-295).
struct Plan {
    int dftW = 0, dftH = 0, hw = 0, blockW = 0, blockH = 0;
    int64_t cost = 0;
};

// Tile grid of one correlation: tiles of blockW x blockH results over the
// rwT x rhT result extent of the template the grid was planned for
// (twL x thL, the bucket maxima for a fleet).
struct TileGeom {
    int ntx = 1, nty = 1;
    int blockW = 1, blockH = 1;
    int rwT = 1, rhT = 1;
    int twL = 1, thL = 1;
    int tileFirst = 0;  // first tile of the launch (plan class)
};

// One plan class: either every tile (no shrunk last band) or the tiles
// above the last band (main), or the last band at the shrunk height.
struct FftClass {
    int n = 0, log2n = 0;    // row transform (dftW)
    int hw = 0, hwp = 0;     // spectrum width and padded row stride
    int dftH = 0, log2H = 0; // column transform
    const float2 *triW = nullptr, *triH = nullptr;
    int tileFirst = 0, ntiles = 0;
};

// Template statistics and the tail constants derived from them.  The raw
// per-channel sums are exact; finalize() derives the rest once the
// effective channel count is known on the device.
struct DevParams {
    unsigned long long tsum[4];   // sum of template bytes per channel
    unsigned long long tsq[4];    // sum of squared bytes per channel
    unsigned int alphaMismatch;   // template alpha plane not constant
    int mode;                     // 0: cn fixed (cnFixed); 1: colour, cn 3/4 by alpha
    int cnFixed;
    int tw, th;
    // derived by k_params_finalize
    int cn;
    int flat;
    long long varSum;
    float templNorm, numScale, varScale;
};

// Per-frame flags written on the device.
struct DevFrame {
    unsigned int alphaMismatch;  // parent alpha plane not constant
    int cnMax;                   // largest effective cn among the members
    int done;                    // CTAs of k_prep finished (last one finalises)
    int normDone;                // CTAs of a solo k_norm finished (last one merges)
};

// One correlation target of the tail kernels: a solo match or one fleet
// member.  tspec is indexed by plan class (0 main, 1 shrunk last band).
// Per-call state is addressed by index (pIdx into the launch's params
// array, the wave slot into the launch's scratch), so a fleet's member
// table is built once per geometry and reused by every call.
struct DevMember {
    const float2 *tspec[2];    // template spectrum, [ch][dftH][hwp], natural rows
    int pIdx;                  // index into the launch's DevParams array
    int tw, th, rw, rh;
    int partBase;              // first partial record of this member (norm CTAs)
    int outIdx;                // result slot
    // region of interest: the result positions [roiX0, roiX1) x [roiY0,
    // roiY1) that take part in the extrema (all of them by default);
    // tiles and row pairs outside it are skipped
    int roiX0, roiY0, roiX1, roiY1;
};

// Where the tail kernels find their targets: a device member table
// (fleets) or one member passed by value (solo matches).
struct MemberSet {
    const DevMember *table;    // nullptr: use `solo`
    DevMember solo;
    int first;                 // first table entry of this launch (wave)
    DevParams *params;
    float2 *scratch[2];        // column-pass output, per wave slot
    size_t scratchStride[2];   // elements between wave slots
    float *map;                // optional score map (solo only)
    float *corr;               // raw correlation, per wave slot (pitch rw), k_norm only
    size_t corrStride;         // elements between wave slots
    float2 *lanes;             // per result (t, den) of the statistics kernel, per wave slot
    size_t lanesStride;        // elements between wave slots
    int anyRoi;                // some member of the launch has a region of interest
    // 0: the reference's arithmetic (per-channel inverses, num = corr - t);
    // 1: the fast form (zero-mean template spectra, channels summed in the
    // frequency domain, one inverse per tile, num = corr); 2: the mixed
    // form (the fast form with its 1024-point inverse rows on the tensor
    // cores).  Nonzero selects the fast form's arithmetic everywhere else.
    int form;
    // Fast-form fleet waves without score maps or regions of interest: the
    // frame's summed-area table of the shared row prefix (ih + 1 rows, the
    // prefix's lanes; all sums modulo 2^32), from which the inverse-rows
    // epilogue forms every window's statistics itself instead of reading
    // den from `lanes` (nullptr: the statistics kernel filled `lanes`).
    const unsigned int *sat;
    size_t satRow;     // u32 per row of the main block (satNp * hp)
    size_t satAlpha;   // u32 offset of the (s3, alpha squares) block; 0: none
    int satNp;         // u32 per x in the main block: 4 (RGBA frame), 2 (gray)
};

struct Partial {
    float minV, maxV;
    long long minI, maxI;
};

// ----------------------------------------------------------- launches
// All launch wrappers queue work on `st` and return the launch status.

cudaError_t launch_gray(const uint8_t *src, long long sstride, int w, int h, uint8_t *dst,
                        long long dstride, cudaStream_t st);
cudaError_t launch_alpha_scan(const uint8_t *img, long long stride, int w, int h,
                              unsigned int *mismatch, cudaStream_t st);
// Template statistics (when tpl is set), parent alpha scan (when parent is
// set) and the finalisation of n params, in one launch.  P (n entries) and
// F must be zeroed, or hold cached template sums, before the launch.
cudaError_t launch_prep(const uint8_t *tpl, long long tstride, int tw, int th, int tstep, int cnStats,
                        const uint8_t *parent, long long pstride, int pw, int ph, DevParams *P, int n,
                        int setInit, int initMode, int initCnFixed, DevFrame *F, cudaStream_t st);
// Forward row pass of every tile of `fc` (or of a template: geometry with
// one 1x1 block whose loads are the template's tw x th).
// Channels [chanFirst, min(chanCount, *cnDev)) are transformed.
// Each sample is pixel * mul - sub[channel] (fixed transform lengths only
// when mul != 1 or sub is set).
cudaError_t launch_fwd_rows(const uint8_t *img, long long istride, int step, int chanCount,
                            const int *cnDev, const TileGeom &g, const FftClass &fc, float2 *spec,
                            int cnS, cudaStream_t st, int chanFirst = 0, const char *label = nullptr,
                            float mul = 1.0f, const float *sub = nullptr,
                            const unsigned long long *subSums = nullptr, float subDiv = 1.0f, int selfSums = 0);
// Column pass.  mode 0: forward only, natural output (template spectra with
// `scale`, fleet frame caches), channels from cnDev; mode 1: forward +
// conj-multiply + inverse, in place on the members' scratch (solo match);
// mode 2: conj-multiply + inverse from a forward frame cache `in` into each
// member's scratch (fleet tails); mode 3: the fast form's channel sum of
// the conj-products, one inverse into the member's single-channel scratch.
// nmembers targets from ms.
cudaError_t launch_cols(int mode, const float2 *in, float2 *out, int cnS, const TileGeom &g,
                        const FftClass &fc, int cls, int chanCount, const int *cnDev, float scale,
                        const MemberSet &ms, int nmembers, cudaStream_t st, const char *label = nullptr);
// Inverse rows + channel accumulation + the correlation-dependent end of
// normOne from the members' lanes, first-occurrence extrema, and the
// member's result written by its last CTA.  Partial records of a member:
// nparts = sum over its plan classes of ntiles * inv_rows_ctas_per_tile;
// partOffset = the records of the classes launched before this one;
// counters[pIdx] must be zero before the first class's launch.  rowsMax
// bounds the result rows of any tile (a single match: the block height;
// a fleet: dftH), the same value for the launch and the partial count.
// wide (fleets in the fast form, whose waves have CTAs to spare): twice
// the row pairs per CTA, no channel accumulator in shared memory.
cudaError_t launch_inv_rows(const TileGeom &g, const FftClass &fc, int cls, int cnS, const MemberSet &ms,
                            int nmembers, int rowsMax, int partOffset, int nparts, Partial *partials, int *counters,
                            cvm_result *out, cudaStream_t st, int wide = 0);
// tc: the launch runs the tensor-core kernel (CVM_FORM_MIXED, 1024-point
// rows), which takes 32 row pairs per CTA in a fleet (wide)
int inv_rows_ctas_per_tile(const FftClass &fc, int rowsMax, int *pairsPerCta, int wide = 0, int tc = 0);
// Normalisation + first-occurrence extrema: CW x B results per CTA, ncx x
// nby CTAs per member, result rows in groups of G; the member's last CTA
// writes its result to out[outIdx].  counters (one int per member of the
// table, or one for a solo match) must be zero before the launch.
struct NormGrid {
    int CW, B, G, ncx, nby, ncCap, cnCap;
    size_t smemBytes;       // dynamic shared memory per CTA
    size_t scratchPerCta;   // unused (kept 0): every shape fits shared memory
};
NormGrid norm_grid(int rwMax, int rhMax, int twMax, int cnCap);
// cnLaunch: the members' effective channel count (kernels are specialised
// on it); a member whose device-side cn differs is skipped by the launch
// and must be covered by the launch for its own cn.
cudaError_t launch_norm(const uint8_t *img, long long istride, int step, const MemberSet &ms, int nmembers,
                        const NormGrid &ng, int cnLaunch, Partial *partials, int *counters, cvm_result *out,
                        cudaStream_t st);
// Separable window statistics: k_hsum writes horizontal window sums (u32,
// interleaved per (row, x): [ih][hp][stat_pitch(cn)] per wave slot),
// k_vstats slides them down BV-row bands and stores per result (t, den)
// into ms.lanes (pitch rw per slot).  One slot takes
// stat_pitch(cnMax) * ih * hp * 4 bytes; [cnMin, cnMax] is the range of
// device-side channel counts the members may have.
struct SepGrid {
    int BV, ncx, nby, hp;
    int rhMax;
};
// u32 slots per (row, x) of the interleaved window-sum / row-prefix
// layouts for cn channels (cn+1 values; 6 for a 4-channel prefix).
constexpr int stat_pitch(int cn) { return cn == 1 ? 2 : (cn <= 3 ? 4 : 8); }
SepGrid sep_grid(int rwMax, int rhMax);
// sharedPrefix: H holds launch_row_prefix's shared planes (no per-member
// k_hsum; each member differences the prefix at its own width).  vst/vev
// (optional): k_vstats runs on vst, ordered after k_hsum by the event vev.
// blk (optional): one match, (ih/16) x hp x stat_pitch(cnMax) u32 for the
// 16-row block sums of H, from which each band starts (tall templates),
// built here; a fleet (sharedPrefix), the block sums of the prefix's main
// block built by launch_vblock.
cudaError_t launch_sep_stats(const uint8_t *img, long long istride, int step, int iw, int ih, const MemberSet &ms,
                             int nmembers, int soloTw, int soloRw, const SepGrid &sg, int cnMin, int cnMax,
                             unsigned int *H, size_t slotStride, cudaStream_t st, int sharedPrefix = 0,
                             cudaStream_t vst = nullptr, cudaEvent_t vev = nullptr, unsigned int *blk = nullptr);
// The 16-row block sums of rows of rowElems u32 (block b = rows 16b ..
// 16b+15, the rows' layout), nblk blocks: a vertical slide starts from them.
cudaError_t launch_vblock(const unsigned int *H, unsigned int *B, int nblk, size_t rowElems, cudaStream_t st);
// Exclusive row prefixes P_q(x, r) (x = 0..iw), u32 modular, interleaved
// [ih][hp][stat_pitch(cnP)] with hp >= iw + 1: the first cnP channel sums
// and the squares of the first min(cnP,3) channels.  For cnP == 4 the main
// block holds (s0, s1, s2, RGB squares) per x ([ih][hp][4]) and a second
// block after it (s3, alpha squares) per x ([ih][hp][2]): 6 * ih * hp u32.
// launch_sep_stats with sharedPrefix reads it with cnMax == cnP.
cudaError_t launch_row_prefix(const uint8_t *img, long long istride, int step, int iw, int ih, int cnP,
                              unsigned int *P, int hp, cudaStream_t st);
// Summed-area table of `rows` rows of rowElems u32 lanes (one block of the
// row prefix): S[y][e] = sum_{r<y} P[r][e], y = 0..rows, modulo 2^32.
// B: scratch of ((rows + 15) / 16 + 1) * rowElems u32.
cudaError_t launch_sat(const unsigned int *P, int rows, size_t rowElems, unsigned int *B, unsigned int *S,
                       cudaStream_t st);

// Stores small host values into device memory through kernel arguments
// (stream ordered, no host buffer lifetime to manage).
cudaError_t upload_bytes(void *dst, const void *src, size_t n, cudaStream_t st);
// rows x rowBytes from device-accessible (page-locked, mapped) host memory
// at src into device memory, by a kernel reading over the host link.
cudaError_t launch_ingest(void *dst, size_t dpitch, const void *src, size_t spitch, size_t rowBytes, int rows,
                          cudaStream_t st);
cudaError_t launch_shrink_gather(const float2 *src, int dftH, float2 *dst, int dh2, int hwp, int cnS,
                                 cudaStream_t st);

// Every occurrence of a score map (the MatchMap recipe of
// cvmatch_test.go:324-381): scratch holds peaks_scratch_ints(w, h) ints;
// *count (device) receives the number of occurrences, xy the first
// maxPeaks of them in raster order as (x, y) pairs.
size_t peaks_scratch_ints(int w, int h);
cudaError_t launch_peaks(const float *map, int w, int h, float thresh, int rx, int ry, int *scratch, int32_t *xy,
                         int maxPeaks, int *count, cudaStream_t st);

// The mixed form's inverse rows on the tensor cores (cvm_tc.cu): applies
// to 1024-point rows of a fused (lanes) launch in CVM_FORM_MIXED; same grid
// and partial records as the FP32 kernel.
struct InvArgs;
bool inv_rows_tc_applies(const FftClass &fc, const MemberSet &ms);
cudaError_t launch_inv_rows_tc(const InvArgs &a, dim3 grid, cudaStream_t st);
cudaError_t tc_selftest(double *dftErr, double *gemmErr);
cudaError_t tc_init();  // the kernel's device tables, once (device set-up)
int tc_error_read_clear();
int rows_error_read_clear();  // the forward rows' TMA waits (cvm_rows.cu)

// kernel-launch counter (exported by cvm_launch_count)
void count_launches(unsigned n);

// Programmatic dependent launch for the calling thread's next launches of
// the transform kernels (rows, columns, inverse rows): each may start its
// CTAs while the preceding kernel of its stream finishes; they wait on the
// device (griddepcontrol.wait) before reading anything.  Only the
// dependency on that preceding kernel is relaxed; event waits stay whole.
void set_pdl(int on);
int pdl_on();
struct PdlScope {
    explicit PdlScope(bool on) { set_pdl(on ? 1 : 0); }
    ~PdlScope() { set_pdl(0); }
};

// sets the calling thread's message returned by cvm_last_error
void set_error_message(const char *msg);

// per-kernel event timing (exported by cvm_profile_enable/cvm_profile_read)
void profile_enable(int on);
int profile_read(int i, char *name, size_t len, double *ms, unsigned long long *count);
int profile_span(int i, char *name, size_t len, double *t0, double *t1);

}  // namespace cvm
