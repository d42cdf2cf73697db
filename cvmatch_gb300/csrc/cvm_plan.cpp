// cvm_plan.cpp -- host-side planning: the tile-geometry argmin, the
// shrunk-band rule, the deterministic twiddle generator and the fleet's
// shape-dominance bucketing.  Pure integer logic except the twiddles,
// which must reproduce the reference's bits: this file is compiled with
// -ffp-contract=off so no multiply-add is ever fused.
#include "cvm_plan.h"

#include <algorithm>
#include <map>

namespace cvm {

int next_pow2(int v) {
    int n = 1;
    while (n < v) n <<= 1;
    return n;
}

int ilog2(int n) {
    int l = 0;
    while ((1 << l) < n) l++;
    return l;
}

// The integer cost-model argmin over power-of-two tile transforms
// (newGoPlan, impl.go:246-295): packed row FFTs, two column passes and a
// linear term, summed over the real tile grid; ties go to the smaller
// transform.  Identical inputs give the identical plan everywhere.
Plan make_plan(int tw, int th, int rw, int rh) {
    const int64_t areaCap = int64_t(1) << 22;
    const int minW = std::max(2, next_pow2(tw)), minH = std::max(2, next_pow2(th));
    const int maxW = std::max(minW, next_pow2(rw + tw - 1));
    const int maxH = std::max(minH, next_pow2(rh + th - 1));
    int bestW = minW, bestH = minH;
    int64_t bestCost = -1, bestArea = 0;
    for (int W = minW; W <= maxW; W <<= 1) {
        for (int H = minH; H <= maxH; H <<= 1) {
            const int64_t area = int64_t(W) * H;
            if (area > areaCap) continue;
            const int bW = std::min(W - tw + 1, rw), bH = std::min(H - th + 1, rh);
            const int64_t ntx = (rw + bW - 1) / bW;
            const int64_t hw = W / 2 + 1;
            const int64_t rowFFT = 5 * int64_t(W) * ilog2(W);
            const int64_t colPass = 5 * int64_t(H) * ilog2(H) * hw;
            const int64_t specN = int64_t(H) * hw;
            // Every band but a ragged last one has height bH, so the
            // per-band sum of the reference's loop collapses to a product
            // (the same integer total, O(1) instead of rh / bH steps).
            auto band = [&](int bh) {
                const int loadH = std::min(bh + th - 1, H);
                return ntx * (int64_t((loadH + 1) / 2 + (bh + 1) / 2) * rowFFT + 2 * colPass + 16 * specN);
            };
            const int64_t full = rh / bH, rest = rh - full * bH;
            int64_t cost = full * band(bH);
            if (rest > 0) cost += band((int)rest);
            if (bestCost < 0 || cost < bestCost || (cost == bestCost && area < bestArea)) {
                bestCost = cost;
                bestArea = area;
                bestW = W;
                bestH = H;
            }
        }
    }
    Plan p;
    p.dftW = bestW;
    p.dftH = bestH;
    p.hw = bestW / 2 + 1;
    p.cost = bestCost;
    p.blockW = std::min(bestW - tw + 1, rw);
    p.blockH = std::min(bestH - th + 1, rh);
    return p;
}

Plan plan_with(int W, int H, int tw, int th, int rw, int rh) {
    Plan p;
    p.dftW = W;
    p.dftH = H;
    p.hw = W / 2 + 1;
    p.blockW = std::min(W - tw + 1, rw);
    p.blockH = std::min(H - th + 1, rh);
    const int64_t ntx = (rw + p.blockW - 1) / p.blockW, nty = (rh + p.blockH - 1) / p.blockH;
    p.cost = ntx * nty * int64_t(W) * H * (ilog2(W) + ilog2(H) + 6);
    return p;
}

// Tile plans the autotuner times for the fast forms (the exact form keeps
// newGoPlan: its bits depend on the plan).  Power-of-two transforms of
// 32 .. 4096 points (the length-specialised kernels) whose blocks hold at
// least 16 results a side, ranked by a GPU cost proxy -- transform points
// x (log2 of the tile size + a per-point memory term) over the tile grid
// -- with newGoPlan's own choice first when it qualifies; at most `count`.
std::vector<Plan> plan_candidates(int tw, int th, int rw, int rh, int count) {
    std::vector<Plan> out;
    const Plan base = make_plan(tw, th, rw, rh);
    auto ok = [&](int W, int H) {
        return W >= 32 && W <= 4096 && H >= 32 && H <= 4096 && int64_t(W) * H <= (int64_t(1) << 22) &&
               std::min(W - tw + 1, rw) >= std::min(16, rw) && std::min(H - th + 1, rh) >= std::min(16, rh) &&
               W - tw + 1 >= 1 && H - th + 1 >= 1;
    };
    if (ok(base.dftW, base.dftH)) out.push_back(plan_with(base.dftW, base.dftH, tw, th, rw, rh));
    std::vector<Plan> all;
    for (int W = 32; W <= 4096; W <<= 1)
        for (int H = 32; H <= 4096; H <<= 1)
            if (ok(W, H) && !(W == base.dftW && H == base.dftH)) all.push_back(plan_with(W, H, tw, th, rw, rh));
    std::stable_sort(all.begin(), all.end(), [](const Plan &a, const Plan &b) {
        return a.cost < b.cost || (a.cost == b.cost && int64_t(a.dftW) * a.dftH < int64_t(b.dftW) * b.dftH);
    });
    for (const Plan &p : all) {
        if ((int)out.size() >= count) break;
        out.push_back(p);
    }
    return out;
}

// The last-band transform height (shrinkDH, impl.go:573-582): 0 when the
// band keeps dftH.
int shrink_dh(const Plan &p, int rh, int th) {
    const int lastY0 = ((rh - 1) / p.blockH) * p.blockH;
    const int lastBh = rh - lastY0;
    if (lastY0 > 0) {
        const int dh2 = std::max(2, next_pow2(lastBh + th - 1));
        if (dh2 < p.dftH) return dh2;
    }
    return 0;
}

int64_t stats_cap(int cn) {
    static const int64_t caps[5] = {0, 11909805, 8421504, 6876129, 5954902};
    return (cn >= 1 && cn <= 4) ? caps[cn] : 0;
}

// cos/sin of pi*j/half by exact dyadic range reduction and the fdlibm
// kernel polynomials (the published __kernel_cos/__kernel_sin minimax
// coefficients), each product rounded before it is added -- the twiddle
// sequence of impl.go:98-133, so tables are identical on every platform.
static void sincospi_frac(int j, int half, float *cs, float *sn) {
    const int m = 2 * j;
    const int k = m / half;
    const int rem = m - k * half;
    double u = double(rem) / double(half);
    bool swap = false;
    if (u > 0.5) {
        u = 1.0 - u;
        swap = true;
    }
    const double y = u * 1.57079632679489661923;
    const double z = y * y;
    double t = z * -1.13596475577881948265e-11;
    t = z * (2.08757232129817482790e-09 + t);
    t = z * (-2.75573143513906633035e-07 + t);
    t = z * (2.48015872894767294178e-05 + t);
    t = z * (-1.38888888888741095749e-03 + t);
    const double r = z * (4.16666666666666019037e-02 + t);
    const double hz = 0.5 * z;
    const double w = 1.0 - hz;
    const double zr = z * r;
    double c = w + (((1.0 - w) - hz) + zr);
    double q = z * 1.58969099521155010221e-10;
    q = z * (-2.50507602534068634195e-08 + q);
    q = z * (2.75573137070700676789e-06 + q);
    q = z * (-1.98412698298579493134e-04 + q);
    const double r2 = 8.33333333332248946124e-03 + q;
    const double v = z * y;
    const double zr2 = z * r2;
    double s = y + v * (-1.66666666666666324348e-01 + zr2);
    if (swap) std::swap(c, s);
    if (k != 0) {
        const double tmp = c;
        c = -s;
        s = tmp;
    }
    *cs = float(c);
    *sn = float(s);
}

// Per-stage radix-4 twiddle triplets (makeTriTwiddles, radix4.go:45-73):
// for quarter size h, w1[j]=cis(-pi j/2h), w2[j]=cis(-pi j/h),
// w3[j]=cis(-3 pi j/2h) with 3j folded into [0,2h) by an exact sign flip.
std::vector<float> tri_twiddles(int n) {
    std::vector<float> tri;
    int h = (ilog2(n) & 1) ? 2 : 1;
    for (; 4 * h <= n; h *= 4) {
        for (int j = 0; j < h; j++) {
            float c, s;
            sincospi_frac(j, 2 * h, &c, &s);
            tri.push_back(c);
            tri.push_back(-s);
        }
        for (int j = 0; j < h; j++) {
            float c, s;
            sincospi_frac(j, h, &c, &s);
            tri.push_back(c);
            tri.push_back(-s);
        }
        for (int j = 0; j < h; j++) {
            int m = 3 * j;
            bool neg = false;
            if (m >= 2 * h) {
                m -= 2 * h;
                neg = true;
            }
            float c, s;
            sincospi_frac(m, 2 * h, &c, &s);
            if (neg) {
                c = -c;
                s = -s;
            }
            tri.push_back(c);
            tri.push_back(-s);
        }
    }
    return tri;
}

// Shape-dominance bucketing (bucketize, fleet.go:111-171): non-flat
// members grouped by power-of-two size class, classes visited largest area
// first and merged into the first bucket that covers them in both axes.
std::vector<Bucket> bucketize(const std::vector<MemberShape> &ms) {
    std::map<std::pair<int, int>, std::vector<int>> byKey;
    std::vector<std::pair<int, int>> keys;
    for (size_t i = 0; i < ms.size(); i++) {
        if (ms[i].flat) continue;
        const std::pair<int, int> k(next_pow2(ms[i].w), next_pow2(ms[i].h));
        auto it = byKey.find(k);
        if (it == byKey.end()) {
            keys.push_back(k);
            byKey[k] = {};
        }
        byKey[k].push_back(int(i));
    }
    std::sort(keys.begin(), keys.end(), [](const std::pair<int, int> &a, const std::pair<int, int> &b) {
        const int64_t aa = int64_t(a.first) * a.second, ab = int64_t(b.first) * b.second;
        if (aa != ab) return aa > ab;
        if (a.first != b.first) return a.first > b.first;
        return a.second > b.second;
    });
    struct Slot {
        int pw2, ph2;
        std::vector<int> members;
    };
    std::vector<Slot> slots;
    for (const auto &k : keys) {
        const std::vector<int> &mem = byKey[k];
        bool placed = false;
        for (Slot &s : slots) {
            if (s.pw2 >= k.first && s.ph2 >= k.second) {
                s.members.insert(s.members.end(), mem.begin(), mem.end());
                placed = true;
                break;
            }
        }
        if (!placed) slots.push_back(Slot{k.first, k.second, mem});
    }
    std::vector<Bucket> out;
    for (Slot &s : slots) {
        std::sort(s.members.begin(), s.members.end());
        Bucket b;
        b.members = s.members;
        for (int mi : s.members) {
            b.tw = std::max(b.tw, ms[mi].w);
            b.th = std::max(b.th, ms[mi].h);
        }
        out.push_back(b);
    }
    return out;
}

}  // namespace cvm
