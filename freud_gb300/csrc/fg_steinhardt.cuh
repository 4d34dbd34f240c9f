// Launch interface of the Steinhardt kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>
#include <vector>

#include "fg_common.cuh"

namespace fg {

constexpr int ST_MAX_L = 31;   // largest spherical-harmonic degree supported
constexpr int ST_MAX_NL = 10;  // largest number of l values per Steinhardt object

// The requested degrees (in the caller's order) and where each one's qlm array
// starts inside one contiguous float2 buffer.
struct StLs
{
    int nl;
    int max_l;
    int l[ST_MAX_NL];
    size_t qlm_offset[ST_MAX_NL]; // in float2 units
    float norm[ST_MAX_NL];        // float(4 pi / (2l + 1))
    int sorted_k[ST_MAX_NL];      // k indices ordered by ascending l
};

void st_upload_tables(cudaStream_t s);
// bond_vd (optional, one float4 per bond): the bond vector box.wrap(p_j - p_i)
// and the bond distance, precomputed per bond (batched frames, where the box
// differs per particle); without it they come from pts, box and dist.
// mean_bonds (optional): bonds per particle, sizes the single-l kernel's work per warp.
// precise: every Y_l^m and the sums over bonds in float-float, each qlm rounded
// once (the Wl path, where the Wigner-3j triple sums cancel); else float32.
void launch_qlm(const DevBox& box, const float* pts, uint32_t n, const uint2* ij, const float* dist,
                const float* weights, const uint32_t* seg, const uint32_t* cnt, const StLs& ls, int weighted,
                float2* qlm, float* ql, cudaStream_t s, const float4* bond_vd = nullptr, double mean_bonds = 0.0,
                int precise = 0);
// bond_j (optional): the neighbour index of each bond, used instead of ij[e].y.
// order (optional): a permutation of the n particles to process them in (e.g. a
// cell grid's slot order, so neighbours' qlm rows are reused from L2); results do
// not depend on it.
void launch_ave(uint32_t n, const uint2* ij, const uint32_t* seg, const uint32_t* cnt, const StLs& ls,
                const float2* qlm, float2* ave, float* ql_ave, cudaStream_t s, const uint32_t* bond_j = nullptr,
                const uint32_t* order = nullptr);
// Wl of every requested l in one launch. The triple sum over m1 + m2 + m3 = 0 is
// taken over classes of terms with equal Re(q_m1 q_m2 q_m3): the permutations of
// (m1, m2, m3) and of (-m1, -m2, -m3) (q_{-m} = (-1)^m conj(q_m), and
// m1 + m2 + m3 = 0). A class is one record (int4): the byte offsets in the row
// (m order 0..l, -1..-l) of its three members (x: first | second << 16, y:
// third), then hi and lo floats of the FP64 sum of the Wigner-3j symbols of the
// class (Wigner3j.cc:22-57 over the same index set). Records of l_k at
// terms + off[k], cnt[k] of them.
struct WlTerms
{
    int off[ST_MAX_NL];
    int cnt[ST_MAX_NL];
};
std::vector<int4> wl_term_classes(int l, double (*w3j)(int, int, int, int));
void launch_wl(uint32_t n, const StLs& ls, const WlTerms& wt, const int4* terms, const float2* src,
               const float* qnorm, int normalize, float* wl, cudaStream_t s);

} // namespace fg
