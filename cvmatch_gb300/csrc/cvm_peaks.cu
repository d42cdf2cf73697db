// cvm_peaks.cu -- every occurrence from a score map, on the device.
//
// The MatchMap recipe of cvmatch_test.go:324-381 (README.md:82-90): a
// result (x, y) is an occurrence when its score is not below the threshold
// and no score within dx in [-rx, rx], dy in [-ry, ry] (clipped to the map)
// is strictly greater.  Occurrences are listed in raster order, so a list
// cut at the caller's capacity keeps the first ones, deterministically.
//
// Three launches: per (row, block of 256 columns) occurrence counts; one
// exclusive scan of those counts in raster order; each block writes its
// occurrences at its scanned offset, ranked within the block by ballots.
#include "cvm_device.cuh"

namespace cvm {
namespace {

constexpr int kPeakCols = 256;

// The recipe's test, with its comparisons: a score that is not below the
// threshold (NaN included) is a candidate, and any strictly greater
// neighbour rejects it.
__device__ __forceinline__ bool is_peak(const float *__restrict__ m, int w, int h, int x, int y, float thresh,
                                        int rx, int ry) {
    const float v = m[(size_t)y * w + x];
    if (v < thresh) return false;
    const int y0 = max(0, y - ry), y1 = min(h - 1, y + ry);
    const int x0 = max(0, x - rx), x1 = min(w - 1, x + rx);
    for (int ny = y0; ny <= y1; ny++) {
        const float *row = m + (size_t)ny * w;
        for (int nx = x0; nx <= x1; nx++)
            if (row[nx] > v) return false;
    }
    return true;
}

__global__ void __launch_bounds__(kPeakCols) k_peaks_count(const float *__restrict__ m, int w, int h, float thresh,
                                                            int rx, int ry, int *counts) {
    __shared__ int wc[kPeakCols / 32];
    const int y = blockIdx.y, x = blockIdx.x * kPeakCols + threadIdx.x;
    const bool p = x < w && is_peak(m, w, h, x, y, thresh, rx, ry);
    const unsigned b = __ballot_sync(0xffffffffu, p);
    if ((threadIdx.x & 31) == 0) wc[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int i = 0; i < kPeakCols / 32; i++) t += wc[i];
        counts[(size_t)y * gridDim.x + blockIdx.x] = t;
    }
}

// Exclusive scan of n counts in place (one CTA of 1024 threads); the total
// goes to *total.
__global__ void __launch_bounds__(1024) k_peaks_scan(int *counts, int n, int *total) {
    __shared__ int part[1024];
    const int tid = threadIdx.x, per = (n + 1023) / 1024;
    const int a = tid * per, b = min(n, a + per);
    int s = 0;
    for (int i = a; i < b; i++) s += counts[i];
    part[tid] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const int v = tid >= o ? part[tid - o] : 0;
        __syncthreads();
        part[tid] += v;
        __syncthreads();
    }
    int run = part[tid] - s;
    for (int i = a; i < b; i++) {
        const int c = counts[i];
        counts[i] = run;
        run += c;
    }
    if (tid == 1023) *total = part[1023];
}

__global__ void __launch_bounds__(kPeakCols) k_peaks_write(const float *__restrict__ m, int w, int h, float thresh,
                                                            int rx, int ry, const int *offsets, int32_t *xy,
                                                            int maxPeaks) {
    __shared__ int wc[kPeakCols / 32];
    const int y = blockIdx.y, x = blockIdx.x * kPeakCols + threadIdx.x;
    const int base = offsets[(size_t)y * gridDim.x + blockIdx.x];
    if (base >= maxPeaks) return;  // uniform per block
    const bool p = x < w && is_peak(m, w, h, x, y, thresh, rx, ry);
    const unsigned b = __ballot_sync(0xffffffffu, p);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wc[warp] = __popc(b);
    __syncthreads();
    int before = 0;
    for (int i = 0; i < warp; i++) before += wc[i];
    if (p) {
        const int idx = base + before + __popc(b & ((1u << lane) - 1u));
        if (idx < maxPeaks) {
            xy[2 * idx] = x;
            xy[2 * idx + 1] = y;
        }
    }
}

}  // namespace

size_t peaks_scratch_ints(int w, int h) { return (size_t)h * ((w + kPeakCols - 1) / kPeakCols); }

cudaError_t launch_peaks(const float *map, int w, int h, float thresh, int rx, int ry, int *scratch, int32_t *xy,
                         int maxPeaks, int *count, cudaStream_t st) {
    const int nxb = (w + kPeakCols - 1) / kPeakCols;
    const dim3 grid(nxb, h);
    {
        ProfScope ps("k_peaks_count", st);
        k_peaks_count<<<grid, kPeakCols, 0, st>>>(map, w, h, thresh, rx, ry, scratch);
    }
    {
        ProfScope ps("k_peaks_scan", st);
        k_peaks_scan<<<1, 1024, 0, st>>>(scratch, nxb * h, count);
    }
    if (maxPeaks > 0) {
        ProfScope ps("k_peaks_write", st);
        k_peaks_write<<<grid, kPeakCols, 0, st>>>(map, w, h, thresh, rx, ry, scratch, xy, maxPeaks);
    }
    count_launches(maxPeaks > 0 ? 3 : 2);
    return cudaGetLastError();
}

}  // namespace cvm
