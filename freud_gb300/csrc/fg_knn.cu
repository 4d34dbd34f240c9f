// k-nearest-neighbour queries (freud/locality/AABBQuery.cc:152-281 and
// LinkCell.cc:575-679): the k points with the smallest r_sq (reference order is by
// distance; ties here are broken by point index), with r_sq < r_max^2 and the
// reference's r_min test (distance >= r_min for AABB arithmetic, r_sq >= r_min^2
// for wrap arithmetic).
//
// k <= 32: warp per query. Candidates from the 27-cell stencil are merged into a
// running top-k held one key per lane (key = r_sq bits << 32 | j), using a 32-wide
// bitonic sort of each candidate chunk and a bitonic merge, with an early skip
// of chunks that cannot improve the current k-th key. A query whose k-th distance
// is not provably inside the stencil (or, in AABB arithmetic, reaches half the
// smallest plane distance where the reference switches to per-point minimum
// images) is handed to the block kernel.
// Block kernel: brute force over all points with the minimum over the 27 images
// per point (AABB) or the wrapped vector, staged and bitonic-sorted in shared memory.
#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int KWARPS = 4;
constexpr int KB_CAP = 8192; // block kernel staging capacity (points)

__device__ __forceinline__ int img_axis_k(int bits, int axis)
{
    return static_cast<int>(static_cast<int8_t>((bits >> (8 * axis)) & 0xff));
}

__device__ __forceinline__ void query_cell_k(const DevBox& b, const DevGrid& g, float4 q, int& cx, int& cy, int& cz,
                                             int& img)
{
    float fx, fy, fz;
    make_fractional(b, q.x, q.y, q.z, fx, fy, fz);
    const float nx = floorf(fx);
    const float ny = floorf(fy);
    const float nz = floorf(fz);
    cx = max(0, min(static_cast<int>(__fsub_rn(fx, nx) * static_cast<float>(g.dim[0])), g.dim[0] - 1));
    cy = max(0, min(static_cast<int>(__fsub_rn(fy, ny) * static_cast<float>(g.dim[1])), g.dim[1] - 1));
    cz = b.is2d ? 0 : max(0, min(static_cast<int>(__fsub_rn(fz, nz) * static_cast<float>(g.dim[2])), g.dim[2] - 1));
    auto cl = [](float n) { return n < -100.0f ? -100 : (n > 100.0f ? 100 : static_cast<int>(n)); };
    img = (cl(nx) & 0xff) | ((cl(ny) & 0xff) << 8) | ((b.is2d ? 0 : cl(nz)) & 0xff) << 16;
}

__device__ __forceinline__ bool pair_vec_k(const DevBox& b, const float (*img)[3], int arith, float4 q, int qimg,
                                           float4 p, int wrap, float& rx, float& ry, float& rz)
{
    if (arith == ARITH_WRAP)
    {
        box_wrap(b, __fsub_rn(p.x, q.x), __fsub_rn(p.y, q.y), __fsub_rn(p.z, q.z), rx, ry, rz);
        return true;
    }
    const int pimg = __float_as_int(p.w);
    const int kx = img_axis_k(pimg, 0) - img_axis_k(qimg, 0) - (wrap % 3 - 1);
    const int ky = img_axis_k(pimg, 1) - img_axis_k(qimg, 1) - ((wrap / 3) % 3 - 1);
    const int kz = img_axis_k(pimg, 2) - img_axis_k(qimg, 2) - (wrap / 9 - 1);
    if (kx < -1 || kx > 1 || ky < -1 || ky > 1 || kz < -1 || kz > 1)
    {
        return false;
    }
    const float* iv = img[(kx + 1) * 9 + (ky + 1) * 3 + (kz + 1)];
    rx = __fsub_rn(p.x, __fadd_rn(q.x, iv[0]));
    ry = __fsub_rn(p.y, __fadd_rn(q.y, iv[1]));
    rz = __fsub_rn(p.z, __fadd_rn(q.z, iv[2]));
    return true;
}

__device__ __forceinline__ bool knn_accept(const KnnParams& p, float rsq)
{
    if (!(rsq < p.r_max_sq))
    {
        return false;
    }
    if (p.arith == ARITH_WRAP)
    {
        return rsq >= p.r_min_sq;
    }
    return __fsqrt_rn(rsq) >= p.r_min;
}

// One compare-exchange stage of a 32-wide bitonic network on (key, payload).
__device__ __forceinline__ void cx_stage(unsigned long long& key, uint32_t& pay, int lane, int j, bool up)
{
    const unsigned long long ok = __shfl_xor_sync(FULL, key, j);
    const uint32_t op = __shfl_xor_sync(FULL, pay, j);
    const bool lower = (lane & j) == 0;
    const bool take = lower ? (up ? ok < key : ok > key) : (up ? ok > key : ok < key);
    if (take)
    {
        key = ok;
        pay = op;
    }
}

__device__ __forceinline__ void sort32(unsigned long long& key, uint32_t& pay, int lane)
{
#pragma unroll
    for (int k = 2; k <= 32; k <<= 1)
    {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            cx_stage(key, pay, lane, j, (lane & k) == 0);
        }
    }
}

// Stencil cells (dx + 1) + 3 (dy + 1) + 9 (dz + 1) ordered by distance class:
// home, 6 faces, 12 edges, 8 corners (2D: home, 4 edges, 4 corners).
__constant__ int c_order3d[27] = {13, 4,  10, 12, 14, 16, 22, 1,  3,  5,  7,  9,  11, 15,
                                  17, 19, 21, 23, 25, 0,  2,  6,  8,  18, 20, 24, 26};
__constant__ int c_order2d[9] = {4, 1, 3, 5, 7, 0, 2, 6, 8};

__global__ void __launch_bounds__(KWARPS * 32)
    k_knn_warp(DevBox b, DevGrid g, const float4* __restrict__ qpos, const uint32_t* __restrict__ qidx, KnnParams p,
               float half_min_plane, uint32_t* __restrict__ tj, float* __restrict__ td, float* __restrict__ tv,
               uint32_t* __restrict__ counts, uint32_t* fail_list, uint32_t* fail_count)
{
    __shared__ float s_img[27][3];
    for (int t = threadIdx.x; t < 81; t += blockDim.x)
    {
        s_img[t / 3][t % 3] = b.img[t / 3][t % 3];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const unsigned long long NONE = ~0ull;
    for (uint32_t t = blockIdx.x * KWARPS + warp; t < p.nq; t += gridDim.x * KWARPS)
    {
        const float4 q = qpos[t];
        const uint32_t qi = qidx[t];
        int cx, cy, cz, qimg;
        query_cell_k(b, g, q, cx, cy, cz, qimg);
        // stencil (same rules as the ball kernels), nearest cells first - home, faces,
        // edges, corners - so the k-th key tightens early and later chunks that
        // cannot improve it are skipped (the result does not depend on the order)
        uint32_t s_start = 0, s_count = 0;
        int s_wrap = 13;
        const int nst = b.is2d ? 9 : 27;
        if (lane < nst)
        {
            const int code = b.is2d ? c_order2d[lane] : c_order3d[lane];
            const int dx = code % 3 - 1;
            const int dy = (code / 3) % 3 - 1;
            const int dz = b.is2d ? 0 : code / 9 - 1;
            auto ok_axis = [&](int d, int dim) {
                if (p.arith == ARITH_AABB || dim >= 3)
                    return true;
                return dim == 1 ? d == 0 : d >= 0;
            };
            if (ok_axis(dx, g.dim[0]) && ok_axis(dy, g.dim[1]) && (b.is2d || ok_axis(dz, g.dim[2])))
            {
                const int ux = cx + dx, uy = cy + dy, uz = cz + dz;
                const int wx = ux < 0 ? -1 : (ux >= g.dim[0] ? 1 : 0);
                const int wy = uy < 0 ? -1 : (uy >= g.dim[1] ? 1 : 0);
                const int wz = uz < 0 ? -1 : (uz >= g.dim[2] ? 1 : 0);
                const int cell = (ux - wx * g.dim[0]) + g.dim[0] * ((uy - wy * g.dim[1]) + g.dim[1] * (uz - wz * g.dim[2]));
                s_start = g.start[cell];
                s_count = g.start[cell + 1] - s_start;
                s_wrap = (wx + 1) + 3 * (wy + 1) + 9 * (wz + 1);
            }
        }
        uint32_t incl = s_count;
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o)
                incl += v;
        }
        const uint32_t s_off = incl - s_count;
        const uint32_t total = __shfl_sync(FULL, incl, 31);

        unsigned long long best = NONE;
        uint32_t bpay = 0;
        for (uint32_t base = 0; base < total; base += 32)
        {
            const uint32_t tt = base + lane;
            const uint32_t tc = tt < total ? tt : total - 1;
            int s = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1)
            {
                const int cand = s + step;
                const uint32_t o = __shfl_sync(FULL, s_off, cand & 31);
                if (cand < 32 && o <= tc)
                    s = cand;
            }
            const uint32_t so = __shfl_sync(FULL, s_off, s);
            const uint32_t ss = __shfl_sync(FULL, s_start, s);
            const int wrap = __shfl_sync(FULL, s_wrap, s);
            const uint32_t slot = ss + (tc - so);
            unsigned long long key = NONE;
            uint32_t pay = 0;
            if (tt < total)
            {
                const float4 pj = g.cpos[slot];
                const uint32_t j = g.cidx[slot];
                float rx, ry, rz;
                if (!(p.exclude_ii && j == qi) && pair_vec_k(b, s_img, p.arith, q, qimg, pj, wrap, rx, ry, rz))
                {
                    const float rsq = dot3(rx, ry, rz);
                    if (knn_accept(p, rsq))
                    {
                        key = (static_cast<unsigned long long>(__float_as_uint(rsq)) << 32) | j;
                        pay = (slot << 5) | static_cast<uint32_t>(wrap);
                    }
                }
            }
            const unsigned long long thr = __shfl_sync(FULL, best, p.k - 1);
            if (__ballot_sync(FULL, key < thr) == 0)
            {
                continue;
            }
            sort32(key, pay, lane);
            // merge: min(best[l], chunk[31-l]) is bitonic and holds the 32 smallest
            const unsigned long long rk = __shfl_sync(FULL, key, 31 - lane);
            const uint32_t rp = __shfl_sync(FULL, pay, 31 - lane);
            if (rk < best)
            {
                best = rk;
                bpay = rp;
            }
#pragma unroll
            for (int j = 16; j > 0; j >>= 1)
            {
                cx_stage(best, bpay, lane, j, true);
            }
        }
        // validity: k-th neighbour provably inside the stencil
        const unsigned long long kth = __shfl_sync(FULL, best, p.k - 1);
        bool valid = true;
        if (kth != NONE)
        {
            const float dk = __fsqrt_rn(__uint_as_float(static_cast<uint32_t>(kth >> 32)));
            if (!(dk < p.covered))
                valid = false;
            if (p.arith == ARITH_AABB && !(dk < half_min_plane))
                valid = false;
        }
        else
        {
            // fewer than k found: fine only if everything within r_max was inside the stencil
            if (!(sqrtf(p.r_max_sq) <= p.covered))
                valid = false;
        }
        if (!valid)
        {
            if (lane == 0)
            {
                fail_list[atomicAdd(fail_count, 1u)] = t;
            }
            continue;
        }
        const uint32_t found = __popc(__ballot_sync(FULL, best != NONE && lane < static_cast<int>(p.k)));
        if (lane < static_cast<int>(p.k) && best != NONE)
        {
            const uint32_t slot = bpay >> 5;
            const int wrap = static_cast<int>(bpay & 31u);
            float rx = 0.f, ry = 0.f, rz = 0.f;
            pair_vec_k(b, s_img, p.arith, q, qimg, g.cpos[slot], wrap, rx, ry, rz);
            const size_t row = static_cast<size_t>(qi) * p.k + lane;
            tj[row] = static_cast<uint32_t>(best & 0xffffffffull);
            td[row] = __fsqrt_rn(dot3(rx, ry, rz));
            tv[3 * row] = rx;
            tv[3 * row + 1] = ry;
            tv[3 * row + 2] = rz;
        }
        if (lane == 0)
        {
            counts[qi] = found;
        }
    }
}

// Thread per query: the query's k nearest candidates of the 27-cell stencil kept
// in registers, unordered, with the position of the current k-th (largest) key;
// a candidate below it replaces it and the largest is found again. Slots k ..
// KMAX - 1 hold key 0, so they are never the largest and never replaced, and the
// first free slot is always the one replaced next (found entries stay in slots
// 0 .. found - 1). Cell-sorted queries put neighbouring queries in one warp: they
// walk nearly the same stencil, reading the same candidates from L1. Validity and
// outputs as k_knn_warp; the rows are ordered afterwards by k_knn_compact.
template<int KMAX>
__global__ void __launch_bounds__(128)
    k_knn_thread(DevBox b, DevGrid g, const float4* __restrict__ qpos, const uint32_t* __restrict__ qidx, KnnParams p,
                 float half_min_plane, uint32_t* __restrict__ tj, float* __restrict__ td, float* __restrict__ tv,
                 uint32_t* __restrict__ counts, uint32_t* fail_list, uint32_t* fail_count)
{
    __shared__ float s_img[27][3];
    for (int t = threadIdx.x; t < 81; t += blockDim.x)
        s_img[t / 3][t % 3] = b.img[t / 3][t % 3];
    __syncthreads();
    const unsigned long long NONE = ~0ull;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < p.nq; t += gridDim.x * blockDim.x)
    {
        const float4 q = qpos[t];
        const uint32_t qi = qidx[t];
        int cx, cy, cz, qimg;
        query_cell_k(b, g, q, cx, cy, cz, qimg);
        unsigned long long key[KMAX];
        uint32_t pay[KMAX];
#pragma unroll
        for (int s = 0; s < KMAX; ++s)
        {
            key[s] = s < static_cast<int>(p.k) ? NONE : 0ull;
            pay[s] = 0;
        }
        unsigned long long worst = NONE;
        int widx = 0;
        const int nst = b.is2d ? 9 : 27;
        for (int c = 0; c < nst; ++c)
        {
            const int code = b.is2d ? c_order2d[c] : c_order3d[c];
            const int dx = code % 3 - 1;
            const int dy = (code / 3) % 3 - 1;
            const int dz = b.is2d ? 0 : code / 9 - 1;
            auto ok_axis = [&](int d, int dim) {
                if (p.arith == ARITH_AABB || dim >= 3)
                    return true;
                return dim == 1 ? d == 0 : d >= 0;
            };
            if (!(ok_axis(dx, g.dim[0]) && ok_axis(dy, g.dim[1]) && (b.is2d || ok_axis(dz, g.dim[2]))))
                continue;
            const int ux = cx + dx, uy = cy + dy, uz = cz + dz;
            const int wx = ux < 0 ? -1 : (ux >= g.dim[0] ? 1 : 0);
            const int wy = uy < 0 ? -1 : (uy >= g.dim[1] ? 1 : 0);
            const int wz = uz < 0 ? -1 : (uz >= g.dim[2] ? 1 : 0);
            const int cell = (ux - wx * g.dim[0]) + g.dim[0] * ((uy - wy * g.dim[1]) + g.dim[1] * (uz - wz * g.dim[2]));
            const int wrap = (wx + 1) + 3 * (wy + 1) + 9 * (wz + 1);
            const uint32_t s0 = g.start[cell], s1 = g.start[cell + 1];
            // AABB arithmetic, candidate inside the box (image 0): k = -n_q - wrap is the
            // cell's, so its validity and image vector are taken once per cell
            const int kx0 = -img_axis_k(qimg, 0) - wx, ky0 = -img_axis_k(qimg, 1) - wy,
                      kz0 = -img_axis_k(qimg, 2) - wz;
            const bool ok0 = kx0 >= -1 && kx0 <= 1 && ky0 >= -1 && ky0 <= 1 && kz0 >= -1 && kz0 <= 1;
            float ivx = 0.f, ivy = 0.f, ivz = 0.f;
            if (ok0)
            {
                const float* iv = s_img[(kx0 + 1) * 9 + (ky0 + 1) * 3 + (kz0 + 1)];
                ivx = iv[0];
                ivy = iv[1];
                ivz = iv[2];
            }
            const float qx = __fadd_rn(q.x, ivx), qy = __fadd_rn(q.y, ivy), qz = __fadd_rn(q.z, ivz);
#pragma unroll 4
            for (uint32_t slot = s0; slot < s1; ++slot)
            {
                const float4 pj = g.cpos[slot];
                const uint32_t j = g.cidx[slot];
                if (p.exclude_ii && j == qi)
                    continue;
                float rx, ry, rz;
                if (p.arith == ARITH_AABB && __float_as_int(pj.w) == 0)
                {
                    if (!ok0)
                        continue;
                    rx = __fsub_rn(pj.x, qx);
                    ry = __fsub_rn(pj.y, qy);
                    rz = __fsub_rn(pj.z, qz);
                }
                else if (!pair_vec_k(b, s_img, p.arith, q, qimg, pj, wrap, rx, ry, rz))
                {
                    continue;
                }
                const float rsq = dot3(rx, ry, rz);
                if (!(rsq < p.r_max_sq))
                    continue;
                // r_min: the square root only when r_min > 0 (sqrt(r^2) >= 0 always holds)
                if (p.arith == ARITH_WRAP ? !(rsq >= p.r_min_sq) : (p.r_min > 0.0f && !(__fsqrt_rn(rsq) >= p.r_min)))
                    continue;
                const unsigned long long kk = (static_cast<unsigned long long>(__float_as_uint(rsq)) << 32) | j;
                if (kk >= worst)
                    continue;
                const uint32_t pp = (slot << 5) | static_cast<uint32_t>(wrap);
                worst = 0ull;
#pragma unroll
                for (int s = 0; s < KMAX; ++s)
                {
                    if (s == widx)
                    {
                        key[s] = kk;
                        pay[s] = pp;
                    }
                }
#pragma unroll
                for (int s = 0; s < KMAX; ++s)
                {
                    if (key[s] > worst)
                    {
                        worst = key[s];
                        widx = s;
                    }
                }
            }
        }
        // validity: k-th neighbour provably inside the stencil
        bool valid = true;
        if (worst != NONE)
        {
            const float dk = __fsqrt_rn(__uint_as_float(static_cast<uint32_t>(worst >> 32)));
            if (!(dk < p.covered))
                valid = false;
            if (p.arith == ARITH_AABB && !(dk < half_min_plane))
                valid = false;
        }
        else if (!(sqrtf(p.r_max_sq) <= p.covered))
        {
            // fewer than k found: fine only if everything within r_max was inside the stencil
            valid = false;
        }
        if (!valid)
        {
            fail_list[atomicAdd(fail_count, 1u)] = t;
            continue;
        }
        uint32_t found = 0;
#pragma unroll
        for (int s = 0; s < KMAX; ++s)
        {
            if (s < static_cast<int>(p.k) && key[s] != NONE)
            {
                const uint32_t slot = pay[s] >> 5;
                const int wrap = static_cast<int>(pay[s] & 31u);
                float rx = 0.f, ry = 0.f, rz = 0.f;
                pair_vec_k(b, s_img, p.arith, q, qimg, g.cpos[slot], wrap, rx, ry, rz);
                const size_t row = static_cast<size_t>(qi) * p.k + found;
                tj[row] = static_cast<uint32_t>(key[s] & 0xffffffffull);
                td[row] = __fsqrt_rn(dot3(rx, ry, rz));
                tv[3 * row] = rx;
                tv[3 * row + 1] = ry;
                tv[3 * row + 2] = rz;
                ++found;
            }
        }
        counts[qi] = found;
    }
}

// Block-wide bitonic sort of key[0, m) with its payload (padded to a power of two
// with the largest key).
__device__ void block_sort_keys(unsigned long long* key, uint32_t* pay, uint32_t m)
{
    uint32_t np = 1;
    while (np < m)
        np <<= 1;
    for (uint32_t e = m + threadIdx.x; e < np; e += blockDim.x)
    {
        key[e] = ~0ull;
        pay[e] = 0;
    }
    __syncthreads();
    for (uint32_t k = 2; k <= np; k <<= 1)
    {
        for (uint32_t j = k >> 1; j > 0; j >>= 1)
        {
            for (uint32_t e = threadIdx.x; e < np; e += blockDim.x)
            {
                const uint32_t pe = e ^ j;
                if (pe > e)
                {
                    const bool up = (e & k) == 0;
                    const unsigned long long a = key[e], c = key[pe];
                    if ((a > c) == up)
                    {
                        key[e] = c;
                        key[pe] = a;
                        const uint32_t tmp = pay[e];
                        pay[e] = pay[pe];
                        pay[pe] = tmp;
                    }
                }
            }
            __syncthreads();
        }
    }
}

// Brute force over all points for the listed queries (t indexes the sorted query
// array). Accepted points stream into a shared buffer of KB_CAP keys (distance,
// index); when a round of blockDim points could overflow it, the buffer is sorted
// and cut to the k best, whose k-th key then filters the rest: the exact k nearest
// for any number of points (k <= KB_CAP / 2).
__global__ void __launch_bounds__(256)
    k_knn_block(DevBox b, const float4* __restrict__ cpos, const uint32_t* __restrict__ cidx, uint32_t n,
                const float4* __restrict__ qpos, const uint32_t* __restrict__ qidx, KnnParams p,
                const uint32_t* __restrict__ list, uint32_t* __restrict__ tj, float* __restrict__ td,
                float* __restrict__ tv, uint32_t* __restrict__ counts, int* err)
{
    extern __shared__ unsigned char smem[];
    unsigned long long* key = reinterpret_cast<unsigned long long*>(smem);
    uint32_t* pay = reinterpret_cast<uint32_t*>(key + KB_CAP);
    __shared__ float s_img[27][3];
    __shared__ uint32_t s_n;
    __shared__ unsigned long long s_thr;
    for (int t = threadIdx.x; t < 81; t += blockDim.x)
    {
        s_img[t / 3][t % 3] = b.img[t / 3][t % 3];
    }
    if (threadIdx.x == 0)
    {
        s_n = 0;
        s_thr = ~0ull;
    }
    __syncthreads();
    if (p.k > static_cast<uint32_t>(KB_CAP / 2))
    {
        if (threadIdx.x == 0)
            atomicExch(err, DEV_CAPACITY);
        return;
    }
    const uint32_t t = list[blockIdx.x];
    const float4 q = qpos[t];
    const uint32_t qi = qidx[t];
    for (uint32_t r0 = 0; r0 < n; r0 += blockDim.x)
    {
        __syncthreads(); // every thread has read the previous round's count
        const uint32_t s = r0 + threadIdx.x;
        const unsigned long long thr = s_thr;
        if (s < n)
        {
            const uint32_t j = cidx[s];
            if (!(p.exclude_ii && j == qi))
            {
                const float4 pj = cpos[s];
                float best = __int_as_float(0x7f800000);
                int bi = 0;
                if (p.arith == ARITH_WRAP)
                {
                    float rx, ry, rz;
                    box_wrap(b, __fsub_rn(pj.x, q.x), __fsub_rn(pj.y, q.y), __fsub_rn(pj.z, q.z), rx, ry, rz);
                    best = dot3(rx, ry, rz);
                }
                else
                {
                    // reference image order: image 0 first, then (i, j, k) lexicographic
                    for (int m = 0; m < 27; ++m)
                    {
                        const int code = m == 0 ? 13 : (m <= 13 ? m - 1 : m);
                        const int kz = code % 3 - 1;
                        if (b.is2d && kz != 0)
                            continue;
                        const float* iv = s_img[code];
                        const float rx = __fsub_rn(pj.x, __fadd_rn(q.x, iv[0]));
                        const float ry = __fsub_rn(pj.y, __fadd_rn(q.y, iv[1]));
                        const float rz = __fsub_rn(pj.z, __fadd_rn(q.z, iv[2]));
                        const float rs = dot3(rx, ry, rz);
                        if (rs < best)
                        {
                            best = rs;
                            bi = code;
                        }
                    }
                }
                const unsigned long long kk = (static_cast<unsigned long long>(__float_as_uint(best)) << 32) | j;
                if (knn_accept(p, best) && kk < thr)
                {
                    const uint32_t e = atomicAdd(&s_n, 1u);
                    key[e] = kk;
                    pay[e] = (s << 5) | static_cast<uint32_t>(bi);
                }
            }
        }
        __syncthreads();
        const uint32_t m = s_n;
        if (m > static_cast<uint32_t>(KB_CAP) - blockDim.x)
        {
            block_sort_keys(key, pay, m);
            if (threadIdx.x == 0)
            {
                const uint32_t kept = m < p.k ? m : p.k;
                s_n = kept;
                if (kept == p.k && kept > 0)
                    s_thr = key[kept - 1];
            }
            __syncthreads();
        }
    }
    const uint32_t m = s_n;
    block_sort_keys(key, pay, m);
    const uint32_t found = m < p.k ? m : p.k;
    for (uint32_t e = threadIdx.x; e < found; e += blockDim.x)
    {
        const uint32_t s = pay[e] >> 5;
        const int code = static_cast<int>(pay[e] & 31u);
        const float4 pj = cpos[s];
        float rx, ry, rz;
        if (p.arith == ARITH_WRAP)
        {
            box_wrap(b, __fsub_rn(pj.x, q.x), __fsub_rn(pj.y, q.y), __fsub_rn(pj.z, q.z), rx, ry, rz);
        }
        else
        {
            const float* iv = s_img[code];
            rx = __fsub_rn(pj.x, __fadd_rn(q.x, iv[0]));
            ry = __fsub_rn(pj.y, __fadd_rn(q.y, iv[1]));
            rz = __fsub_rn(pj.z, __fadd_rn(q.z, iv[2]));
        }
        const size_t row = static_cast<size_t>(qi) * p.k + e;
        tj[row] = static_cast<uint32_t>(key[e] & 0xffffffffull);
        td[row] = __fsqrt_rn(dot3(rx, ry, rz));
        tv[3 * row] = rx;
        tv[3 * row + 1] = ry;
        tv[3 * row + 2] = rz;
    }
    if (threadIdx.x == 0)
        counts[qi] = found;
}

// Thread per query, rows of at most KMAX entries held in registers: each entry's
// rank in the row's order (by j, or by distance then j; keys are distinct) is
// the number of smaller keys, and the entry is written at that rank.
template<int KMAX>
__global__ void __launch_bounds__(128)
    k_knn_compact_reg(const uint32_t* __restrict__ tj, const float* __restrict__ td, const float* __restrict__ tv,
                      uint32_t k, uint32_t nq, const uint32_t* __restrict__ counts,
                      const uint64_t* __restrict__ offsets, int by_distance, uint2* __restrict__ ij,
                      float* __restrict__ dist, float* __restrict__ vec)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    {
        const uint32_t c = counts[i];
        const size_t row = static_cast<size_t>(i) * k;
        const uint64_t off = offsets[i];
        uint64_t key[KMAX];
#pragma unroll
        for (int x = 0; x < KMAX; ++x)
        {
            key[x] = ~0ull;
            if (static_cast<uint32_t>(x) < c)
            {
                const uint32_t j = tj[row + x];
                const uint32_t db = __float_as_uint(td[row + x]);
                key[x] = by_distance ? ((static_cast<uint64_t>(db) << 32) | j) : ((static_cast<uint64_t>(j) << 32) | db);
            }
        }
#pragma unroll
        for (int x = 0; x < KMAX; ++x)
        {
            if (static_cast<uint32_t>(x) < c)
            {
                uint32_t r = 0;
#pragma unroll
                for (int y = 0; y < KMAX; ++y)
                    r += key[y] < key[x] ? 1u : 0u;
                const uint64_t o = off + r;
                const uint32_t j = by_distance ? static_cast<uint32_t>(key[x]) : static_cast<uint32_t>(key[x] >> 32);
                const uint32_t db = by_distance ? static_cast<uint32_t>(key[x] >> 32) : static_cast<uint32_t>(key[x]);
                ij[o] = make_uint2(i, j);
                dist[o] = __uint_as_float(db);
                vec[3 * o] = tv[3 * (row + x)];
                vec[3 * o + 1] = tv[3 * (row + x) + 1];
                vec[3 * o + 2] = tv[3 * (row + x) + 2];
            }
        }
    }
}

// Thread per query: order its row (by j, or by distance then j) and copy it out.
__global__ void k_knn_compact(const uint32_t* __restrict__ tj, const float* __restrict__ td,
                              const float* __restrict__ tv, uint32_t k, uint32_t nq, const uint32_t* __restrict__ counts,
                              const uint64_t* __restrict__ offsets, int by_distance, uint2* __restrict__ ij,
                              float* __restrict__ dist, float* __restrict__ vec)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    {
        const uint32_t c = counts[i];
        const size_t row = static_cast<size_t>(i) * k;
        const uint64_t off = offsets[i];
        // selection of the next smallest remaining entry (rows are short)
        uint64_t done_key = 0;
        bool first = true;
        for (uint32_t e = 0; e < c; ++e)
        {
            uint64_t best = ~0ull;
            uint32_t bi = 0;
            for (uint32_t x = 0; x < c; ++x)
            {
                const uint32_t j = tj[row + x];
                const uint64_t key = by_distance
                    ? ((static_cast<uint64_t>(__float_as_uint(td[row + x])) << 32) | j)
                    : ((static_cast<uint64_t>(j) << 32) | __float_as_uint(td[row + x]));
                if ((first || key > done_key) && key < best)
                {
                    best = key;
                    bi = x;
                }
            }
            first = false;
            done_key = best;
            ij[off + e] = make_uint2(i, tj[row + bi]);
            dist[off + e] = td[row + bi];
            vec[3 * (off + e)] = tv[3 * (row + bi)];
            vec[3 * (off + e) + 1] = tv[3 * (row + bi) + 1];
            vec[3 * (off + e) + 2] = tv[3 * (row + bi) + 2];
        }
    }
}

} // namespace

void launch_knn_warp(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                     const KnnParams& p, uint32_t* tj, float* td, float* tv, uint32_t* counts, uint32_t* fail_list,
                     uint32_t* fail_count, cudaStream_t s)
{
    if (p.nq == 0)
        return;
    // half of the smallest nearest-plane distance (host computes it into covered's sibling)
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t want = (p.nq + KWARPS - 1) / KWARPS;
    const uint32_t cap = static_cast<uint32_t>(sms) * 16;
    float pd0 = box.L[0] / sqrtf(1.0f + box.xy * box.xy + (box.xy * box.yz - box.xz) * (box.xy * box.yz - box.xz));
    float pd1 = box.L[1] / sqrtf(1.0f + box.yz * box.yz);
    float mp = fminf(pd0, pd1);
    if (!box.is2d)
        mp = fminf(mp, box.L[2]);
    if (p.k <= 16)
    {
        // thread per query (cell-sorted queries: a warp walks nearly one stencil)
        const uint32_t blocks = (p.nq + 127) / 128;
        ProfScope prof_("k_knn_thread", s);
        if (p.k <= 8)
            k_knn_thread<8><<<blocks, 128, 0, s>>>(box, g, qpos, qidx, p, mp / 2.0f, tj, td, tv, counts, fail_list,
                                                   fail_count);
        else if (p.k <= 12)
            k_knn_thread<12><<<blocks, 128, 0, s>>>(box, g, qpos, qidx, p, mp / 2.0f, tj, td, tv, counts, fail_list,
                                                    fail_count);
        else
            k_knn_thread<16><<<blocks, 128, 0, s>>>(box, g, qpos, qidx, p, mp / 2.0f, tj, td, tv, counts, fail_list,
                                                    fail_count);
    }
    else
    {
        ProfScope prof_("k_knn_warp", s);
        k_knn_warp<<<want < cap ? want : cap, KWARPS * 32, 0, s>>>(box, g, qpos, qidx, p, mp / 2.0f, tj, td, tv, counts,
                                                                   fail_list, fail_count);
    }
}

size_t knn_block_capacity()
{
    return KB_CAP;
}

void launch_knn_block(const DevBox& box, const float4* cpos, const uint32_t* cidx, uint32_t n, const float4* qpos,
                       const uint32_t* qidx, const KnnParams& p, const uint32_t* list, uint32_t nlist, uint32_t* tj,
                       float* td, float* tv, uint32_t* counts, int* err, cudaStream_t s)
{
    if (nlist == 0)
        return;
    const size_t smem = static_cast<size_t>(KB_CAP) * (sizeof(unsigned long long) + sizeof(uint32_t));
    static bool configured = false;
    if (!configured)
    {
        cudaFuncSetAttribute(k_knn_block, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        configured = true;
    }
    {
        ProfScope prof_("k_knn_block", s);
        k_knn_block<<<nlist, 256, smem, s>>>(box, cpos, cidx, n, qpos, qidx, p, list, tj, td, tv, counts, err);
    }
}

void launch_knn_compact(const uint32_t* tj, const float* td, const float* tv, uint32_t k, uint32_t nq,
                        const uint32_t* counts, const uint64_t* offsets, int by_distance, uint2* ij, float* dist,
                        float* vec, cudaStream_t s)
{
    if (nq == 0)
        return;
    const uint32_t blocks = (nq + 127) / 128;
    if (k <= 16)
    {
        ProfScope prof_("k_knn_compact", s);
        const uint32_t b = blocks < 152 * 64 ? blocks : 152 * 64;
        if (k <= 12)
            k_knn_compact_reg<12><<<b, 128, 0, s>>>(tj, td, tv, k, nq, counts, offsets, by_distance, ij, dist, vec);
        else
            k_knn_compact_reg<16><<<b, 128, 0, s>>>(tj, td, tv, k, nq, counts, offsets, by_distance, ij, dist, vec);
        return;
    }
    {
        ProfScope prof_("k_knn_compact", s);
        k_knn_compact<<<blocks < 152 * 64 ? blocks : 152 * 64, 128, 0, s>>>(tj, td, tv, k, nq, counts, offsets,
                                                                          by_distance, ij, dist, vec);
    }
}

} // namespace fg
