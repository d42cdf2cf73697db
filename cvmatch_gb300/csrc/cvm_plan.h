// cvm_plan.h -- host-side planning (see cvm_plan.cpp).
#pragma once

#include <cstdint>
#include <vector>

#include "cvm_internal.h"

namespace cvm {

int next_pow2(int v);
int ilog2(int n);
Plan make_plan(int tw, int th, int rw, int rh);
// A plan with the given transform sizes (blocks as newGoPlan forms them).
Plan plan_with(int W, int H, int tw, int th, int rw, int rh);
// The autotuner's candidate plans for the fast forms (see cvm_plan.cpp).
std::vector<Plan> plan_candidates(int tw, int th, int rw, int rh, int count);
int shrink_dh(const Plan &p, int rh, int th);
int64_t stats_cap(int cn);
std::vector<float> tri_twiddles(int n);

struct MemberShape {
    int w, h;
    bool flat;
};

struct Bucket {
    int tw = 0, th = 0;
    std::vector<int> members;  // global member indices, ascending
};

std::vector<Bucket> bucketize(const std::vector<MemberShape> &ms);

}  // namespace cvm
