// Device-side NeighborList construction helpers: bonds from user arrays
// (NeighborList.cc:51-82), all pairs (NeighborList.cc:84-128), filtering
// (NeighborList.cc:234-307) and find_first_index (NeighborList.cc:309-316, 417-428).
#include "fg_nlist.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

int blocks_for(uint64_t n, int threads)
{
    uint64_t b = (n + threads - 1) / threads;
    const uint64_t cap = 152ull * 64ull;
    return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}

// distance = sqrt(dot(v, v)) (NeighborBond.h:40-43), 4-argument NeighborBond ctor.
__global__ void k_from_arrays(const uint32_t* __restrict__ qi, const uint32_t* __restrict__ pi,
                              const float* __restrict__ vec, uint64_t nb, uint2* __restrict__ ij,
                              float* __restrict__ dist)
{
    for (uint64_t b = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; b < nb; b += (uint64_t) gridDim.x * blockDim.x)
    {
        ij[b] = make_uint2(qi[b], pi[b]);
        dist[b] = __fsqrt_rn(dot3(vec[3 * b], vec[3 * b + 1], vec[3 * b + 2]));
    }
}

// All pairs: bond (i, j) at i * np + j (minus the skipped diagonal), vector
// box.wrap(query_points[i] - points[j]) as the reference computes it.
__global__ void k_all_pairs(DevBox b, const float* __restrict__ pts, uint32_t np, const float* __restrict__ qpts,
                            uint32_t nq, int exclude_ii, uint64_t nb, uint2* __restrict__ ij, float* __restrict__ dist,
                            float* __restrict__ vec)
{
    for (uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; t < static_cast<uint64_t>(nq) * np;
         t += (uint64_t) gridDim.x * blockDim.x)
    {
        const uint32_t i = static_cast<uint32_t>(t / np);
        const uint32_t j = static_cast<uint32_t>(t % np);
        if (exclude_ii && i == j)
        {
            continue;
        }
        // NeighborList.cc:107-123: row i starts at i * np - min(i, np) when excluding i == j
        const uint64_t base = static_cast<uint64_t>(i) * np - (exclude_ii ? (i < np ? i : np) : 0u);
        const uint64_t bond = base + j - ((exclude_ii && i < np && j > i) ? 1u : 0u);
        float rx, ry, rz;
        box_wrap(b, __fsub_rn(qpts[3 * (size_t) i], pts[3 * (size_t) j]),
                 __fsub_rn(qpts[3 * (size_t) i + 1], pts[3 * (size_t) j + 1]),
                 __fsub_rn(qpts[3 * (size_t) i + 2], pts[3 * (size_t) j + 2]), rx, ry, rz);
        if (bond < nb)
        {
            ij[bond] = make_uint2(i, j);
            dist[bond] = __fsqrt_rn(dot3(rx, ry, rz));
            vec[3 * bond] = rx;
            vec[3 * bond + 1] = ry;
            vec[3 * bond + 2] = rz;
        }
    }
}

__global__ void k_keep_r(const float* __restrict__ dist, uint64_t nb, float r_max, float r_min, uint32_t* keep)
{
    for (uint64_t b = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; b < nb; b += (uint64_t) gridDim.x * blockDim.x)
    {
        keep[b] = (dist[b] >= r_min && dist[b] < r_max) ? 1u : 0u;
    }
}

__global__ void k_keep_u8(const uint8_t* __restrict__ in, uint64_t nb, uint32_t* keep)
{
    for (uint64_t b = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; b < nb; b += (uint64_t) gridDim.x * blockDim.x)
    {
        keep[b] = in[b] != 0 ? 1u : 0u;
    }
}

__global__ void k_compact(const uint32_t* __restrict__ keep, const uint64_t* __restrict__ pos, uint64_t nb,
                          const uint2* __restrict__ ij, const float* __restrict__ dist, const float* __restrict__ w,
                          const float* __restrict__ vec, uint2* __restrict__ ij2, float* __restrict__ dist2,
                          float* __restrict__ w2, float* __restrict__ vec2)
{
    for (uint64_t b = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; b < nb; b += (uint64_t) gridDim.x * blockDim.x)
    {
        if (keep[b])
        {
            const uint64_t o = pos[b];
            ij2[o] = ij[b];
            dist2[o] = dist[b];
            if (w != nullptr)
            {
                w2[o] = w[b];
            }
            vec2[3 * o] = vec[3 * b];
            vec2[3 * o + 1] = vec[3 * b + 1];
            vec2[3 * o + 2] = vec[3 * b + 2];
        }
    }
}

// Lowest bond index whose query index is >= i.
__global__ void k_first_index(const uint2* __restrict__ ij, uint64_t nb, uint32_t i, uint64_t* out)
{
    uint64_t lo = 0, hi = nb;
    while (lo < hi)
    {
        const uint64_t mid = (lo + hi) / 2;
        if (ij[mid].x < i)
        {
            lo = mid + 1;
        }
        else
        {
            hi = mid;
        }
    }
    *out = lo;
}

} // namespace

void launch_from_arrays(const uint32_t* qi, const uint32_t* pi, const float* vec, uint64_t nb, uint2* ij, float* dist,
                        cudaStream_t s)
{
    if (nb == 0)
        return;
    {
        ProfScope prof_("k_from_arrays", s);
        k_from_arrays<<<blocks_for(nb, 256), 256, 0, s>>>(qi, pi, vec, nb, ij, dist);
    }
}

void launch_all_pairs(const DevBox& b, const float* pts, uint32_t np, const float* qpts, uint32_t nq, int exclude_ii,
                      uint64_t nb, uint2* ij, float* dist, float* vec, cudaStream_t s)
{
    if (nb == 0)
        return;
    {
        ProfScope prof_("k_all_pairs", s);
        k_all_pairs<<<blocks_for(static_cast<uint64_t>(nq) * np, 256), 256, 0, s>>>(b, pts, np, qpts, nq, exclude_ii, nb,
                                                                                  ij, dist, vec);
    }
}

void launch_keep_r(const float* dist, uint64_t nb, float r_max, float r_min, uint32_t* keep, cudaStream_t s)
{
    if (nb == 0)
        return;
    {
        ProfScope prof_("k_keep_r", s);
        k_keep_r<<<blocks_for(nb, 256), 256, 0, s>>>(dist, nb, r_max, r_min, keep);
    }
}

void launch_keep_u8(const uint8_t* in, uint64_t nb, uint32_t* keep, cudaStream_t s)
{
    if (nb == 0)
        return;
    {
        ProfScope prof_("k_keep_u8", s);
        k_keep_u8<<<blocks_for(nb, 256), 256, 0, s>>>(in, nb, keep);
    }
}

void launch_compact(const uint32_t* keep, const uint64_t* pos, uint64_t nb, const uint2* ij, const float* dist,
                    const float* w, const float* vec, uint2* ij2, float* dist2, float* w2, float* vec2, cudaStream_t s)
{
    if (nb == 0)
        return;
    {
        ProfScope prof_("k_compact", s);
        k_compact<<<blocks_for(nb, 256), 256, 0, s>>>(keep, pos, nb, ij, dist, w, vec, ij2, dist2, w2, vec2);
    }
}

void launch_first_index(const uint2* ij, uint64_t nb, uint32_t i, uint64_t* out, cudaStream_t s)
{
    {
        ProfScope prof_("k_first_index", s);
        k_first_index<<<1, 1, 0, s>>>(ij, nb, i, out);
    }
}

} // namespace fg
