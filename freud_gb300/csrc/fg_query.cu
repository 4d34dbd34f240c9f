// Ball queries: warp-per-query traversal of the 27-cell (9 in 2D) stencil with
// exact float32 pair arithmetic, in three modes:
//   COUNT - bonds per query (first pass of NeighborList construction)
//   EMIT  - bonds written at the query's offset in reference order: sorted by
//           (i, j, weight, distance) or (i, distance, j, weight)
//           (NeighborQuery.h:434-481, NeighborBond.h:80-117), via warp-aggregated
//           compaction into shared memory and a warp bitonic sort
//   HIST  - fused RDF binning (RDF.cc:101-110, Histogram.h:152-174) into
//           block-private shared-memory histograms flushed with 64-bit atomics
//
// Pair arithmetic (selected per query object):
//   AABB  r = p_j - (q + image_k)  (AABBQuery.cc:93,125), image_k the reference
//         image vector (NeighborQuery.h:546-560) for k = n_j - n_q - wrap, where
//         n is the integer box image of each point and wrap the cell wrap count;
//         only |k| <= 1 per axis is tested, as the reference only has 27 images.
//   WRAP  r = box.wrap(p_j - q)    (LinkCell.cc:522), over distinct wrapped cells.
// Accept: r_sq < r_max^2 && r_sq >= r_min^2, exclude_ii by index.
#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

enum Mode
{
    MODE_COUNT = 0,
    MODE_EMIT = 1,
    MODE_HIST = 2,
};

constexpr int QWARPS = 4; // warps per block in the query kernels
constexpr unsigned FULL = 0xffffffffu;
constexpr int HIST_SMEM_BINS = 4096;
constexpr int HIST_COPIES = 2; // privatised copies per block (warp w uses copy w % HIST_COPIES)

__device__ __forceinline__ int img_axis(int bits, int axis)
{
    return static_cast<int>(static_cast<int8_t>((bits >> (8 * axis)) & 0xff));
}

// One stencil item per lane: a neighbour cell (with its wrap counts) of the query's cell.
struct Stencil
{
    uint32_t start; // first sorted slot of the cell
    uint32_t count; // candidates contributed by this lane
    int wrap;       // packed wrap counts (wx+1) + 3*(wy+1) + 9*(wz+1)
    uint32_t off;   // exclusive prefix of counts over lanes
    uint32_t total; // warp-uniform number of candidates
};

__device__ __forceinline__ void query_cell(const DevBox& b, const DevGrid& g, float4 q, int& cx, int& cy, int& cz,
                                           int& img)
{
    if (g.ghost)
    {
        // ghost grid: axis-aligned cell, cx = -1 outside the grid (no bonds,
        // CellIterator.h:52-57)
        const float fx = floorf(__fmul_rn(__fsub_rn(q.x, g.gmin[0]), g.ginv));
        const float fy = floorf(__fmul_rn(__fsub_rn(q.y, g.gmin[1]), g.ginv));
        const float fz = floorf(__fmul_rn(__fsub_rn(q.z, g.gmin[2]), g.ginv));
        img = 0;
        if (fx >= 0.0f && fy >= 0.0f && fz >= 0.0f && fx < static_cast<float>(g.dim[0])
            && fy < static_cast<float>(g.dim[1]) && fz < static_cast<float>(g.dim[2]))
        {
            cx = static_cast<int>(fx);
            cy = static_cast<int>(fy);
            cz = static_cast<int>(fz);
        }
        else
        {
            cx = cy = cz = -1;
        }
        return;
    }
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

// Whether offset d along an axis of dim cells is visited (wrap arithmetic visits
// each distinct wrapped cell once; AABB arithmetic visits every (cell, wrap) pair).
__device__ __forceinline__ bool offset_ok(int d, int dim, int arith)
{
    if (arith == ARITH_AABB || dim >= 3)
    {
        return true;
    }
    if (dim == 1)
    {
        return d == 0;
    }
    return d >= 0; // dim == 2: cells c and c+1 (mod 2)
}

__device__ __forceinline__ Stencil build_stencil(const DevBox& b, const DevGrid& g, int cx, int cy, int cz, int arith,
                                                 int lane)
{
    Stencil st;
    st.start = 0;
    st.count = 0;
    st.wrap = 13;
    const int nst = b.is2d ? 9 : 27;
    if (arith == ARITH_GHOST)
    {
        // no wrap: the 27 neighbours clipped to the grid; none for a query outside it
        if (lane < 27 && cx >= 0)
        {
            const int ux = cx + lane % 3 - 1;
            const int uy = cy + (lane / 3) % 3 - 1;
            const int uz = cz + lane / 9 - 1;
            if (ux >= 0 && uy >= 0 && uz >= 0 && ux < g.dim[0] && uy < g.dim[1] && uz < g.dim[2])
            {
                const int cell = ux + g.dim[0] * (uy + g.dim[1] * uz);
                st.start = g.start[cell];
                st.count = g.start[cell + 1] - st.start;
            }
        }
    }
    else if (lane < nst)
    {
        const int dx = lane % 3 - 1;
        const int dy = (lane / 3) % 3 - 1;
        const int dz = b.is2d ? 0 : lane / 9 - 1;
        if (offset_ok(dx, g.dim[0], arith) && offset_ok(dy, g.dim[1], arith)
            && (b.is2d || offset_ok(dz, g.dim[2], arith)))
        {
            const int ux = cx + dx;
            const int uy = cy + dy;
            const int uz = cz + dz;
            const int wx = ux < 0 ? -1 : (ux >= g.dim[0] ? 1 : 0);
            const int wy = uy < 0 ? -1 : (uy >= g.dim[1] ? 1 : 0);
            const int wz = uz < 0 ? -1 : (uz >= g.dim[2] ? 1 : 0);
            const int ccx = ux - wx * g.dim[0];
            const int ccy = uy - wy * g.dim[1];
            const int ccz = uz - wz * g.dim[2];
            const int cell = ccx + g.dim[0] * (ccy + g.dim[1] * ccz);
            st.start = g.start[cell];
            st.count = g.start[cell + 1] - st.start;
            st.wrap = (wx + 1) + 3 * (wy + 1) + 9 * (wz + 1);
        }
    }
    uint32_t incl = st.count;
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t t = __shfl_up_sync(FULL, incl, o);
        if (lane >= o)
        {
            incl += t;
        }
    }
    st.off = incl - st.count;
    st.total = __shfl_sync(FULL, incl, 31);
    return st;
}

// Locate candidate t (< total) in the stencil: returns the sorted slot and the wrap code.
__device__ __forceinline__ void locate(const Stencil& st, uint32_t t, uint32_t& slot, int& wrap)
{
    int s = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1)
    {
        const int cand = s + step;
        const uint32_t o = __shfl_sync(FULL, st.off, cand & 31);
        if (cand < 32 && o <= t)
        {
            s = cand;
        }
    }
    const uint32_t so = __shfl_sync(FULL, st.off, s);
    const uint32_t ss = __shfl_sync(FULL, st.start, s);
    wrap = __shfl_sync(FULL, st.wrap, s);
    slot = ss + (t - so);
}

// Exact pair vector. Returns false if the candidate cannot be a bond through the
// tested image (AABB arithmetic with |k| > 1).
__device__ __forceinline__ bool pair_vector(const DevBox& b, const float (*img)[3], int arith, float4 q, int qimg,
                                            float4 p, int wrap, float& rx, float& ry, float& rz)
{
    if (arith == ARITH_WRAP)
    {
        box_wrap(b, __fsub_rn(p.x, q.x), __fsub_rn(p.y, q.y), __fsub_rn(p.z, q.z), rx, ry, rz);
        return true;
    }
    if (arith == ARITH_GHOST)
    {
        rx = __fsub_rn(p.x, q.x);
        ry = __fsub_rn(p.y, q.y);
        rz = __fsub_rn(p.z, q.z);
        return true;
    }
    const int pimg = __float_as_int(p.w);
    const int kx = img_axis(pimg, 0) - img_axis(qimg, 0) - (wrap % 3 - 1);
    const int ky = img_axis(pimg, 1) - img_axis(qimg, 1) - ((wrap / 3) % 3 - 1);
    const int kz = img_axis(pimg, 2) - img_axis(qimg, 2) - (wrap / 9 - 1);
    if (kx < -1 || kx > 1 || ky < -1 || ky > 1 || kz < -1 || kz > 1)
    {
        return false;
    }
    const float* iv = img[(kx + 1) * 9 + (ky + 1) * 3 + (kz + 1)];
    const float qx = __fadd_rn(q.x, iv[0]);
    const float qy = __fadd_rn(q.y, iv[1]);
    const float qz = __fadd_rn(q.z, iv[2]);
    rx = __fsub_rn(p.x, qx);
    ry = __fsub_rn(p.y, qy);
    rz = __fsub_rn(p.z, qz);
    return true;
}

struct WarpStage
{
    unsigned long long key[EMIT_CAP];
    float4 val[EMIT_CAP]; // (vx, vy, vz, d)
    unsigned short slot[EMIT_CAP];
};

// Warp bitonic sort of n keys (n <= EMIT_CAP) in shared memory with a slot payload.
__device__ void warp_sort(unsigned long long* key, unsigned short* slot, int n, int lane)
{
    int np = 32;
    while (np < n)
    {
        np <<= 1;
    }
    for (int e = n + lane; e < np; e += 32)
    {
        key[e] = ~0ull;
        slot[e] = 0;
    }
    __syncwarp();
    for (int k = 2; k <= np; k <<= 1)
    {
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int e = lane; e < np; e += 32)
            {
                const int p = e ^ j;
                if (p > e)
                {
                    const bool up = (e & k) == 0;
                    const unsigned long long a = key[e];
                    const unsigned long long c = key[p];
                    if ((a > c) == up)
                    {
                        key[e] = c;
                        key[p] = a;
                        const unsigned short t = slot[e];
                        slot[e] = slot[p];
                        slot[p] = t;
                    }
                }
            }
            __syncwarp();
        }
    }
}

__device__ __forceinline__ unsigned long long order_key(int by_distance, uint32_t j, float d)
{
    // distances are >= 0, so their bit patterns order like the values
    return by_distance ? ((static_cast<unsigned long long>(__float_as_uint(d)) << 32) | j)
                       : ((static_cast<unsigned long long>(j) << 32) | __float_as_uint(d));
}

template<int MODE>
__global__ void __launch_bounds__(QWARPS * 32)
    k_ball(DevBox b, DevGrid g, const float4* __restrict__ qpos, const uint32_t* __restrict__ qidx, BallParams p,
           uint32_t* __restrict__ counts, const uint64_t* __restrict__ offsets, int by_distance, uint2* __restrict__ ij,
           float* __restrict__ dist, float* __restrict__ vec, uint32_t* heavy_list, uint32_t* heavy_count, int* err,
           HistParams h, unsigned long long* __restrict__ hist, const uint32_t* __restrict__ list)
{
    __shared__ float s_img[27][3];
    __shared__ WarpStage s_stage[MODE == MODE_EMIT ? QWARPS : 1];
    __shared__ unsigned int s_hist[MODE == MODE_HIST ? HIST_COPIES * HIST_SMEM_BINS : 1];

    for (int t = threadIdx.x; t < 81; t += blockDim.x)
    {
        s_img[t / 3][t % 3] = b.img[t / 3][t % 3];
    }
    const bool smem_hist = MODE == MODE_HIST && h.bins <= HIST_SMEM_BINS;
    if (MODE == MODE_HIST && smem_hist)
    {
        for (int t = threadIdx.x; t < HIST_COPIES * static_cast<int>(h.bins); t += blockDim.x)
        {
            s_hist[(t / h.bins) * HIST_SMEM_BINS + t % h.bins] = 0;
        }
    }
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    unsigned int* my_hist = s_hist + (warp % HIST_COPIES) * HIST_SMEM_BINS;

    for (uint32_t tl = blockIdx.x * QWARPS + warp; tl < p.nq; tl += gridDim.x * QWARPS)
    {
        const uint32_t t = list != nullptr ? list[tl] : tl;
        const float4 q = qpos[t];
        const uint32_t qi = qidx[t];
        if (MODE == MODE_EMIT)
        {
            const uint32_t c = counts[qi];
            if (c > EMIT_CAP)
            {
                if (lane == 0)
                {
                    heavy_list[atomicAdd(heavy_count, 1u)] = t;
                }
                continue;
            }
            if (c == 0)
            {
                continue;
            }
        }
        int cx, cy, cz, qimg;
        query_cell(b, g, q, cx, cy, cz, qimg);
        const Stencil st = build_stencil(b, g, cx, cy, cz, p.arith, lane);
        uint32_t found = 0;
        for (uint32_t base = 0; base < st.total; base += 32)
        {
            const uint32_t tt = base + lane;
            bool ok = false;
            float rx = 0.f, ry = 0.f, rz = 0.f, rsq = 0.f;
            uint32_t j = 0;
            uint32_t slot;
            int wrap;
            locate(st, tt < st.total ? tt : st.total - 1, slot, wrap); // warp-uniform shuffles
            if (tt < st.total)
            {
                const float4 pj = g.cpos[slot];
                j = g.cidx[slot];
                if (!(p.exclude_ii && j == qi) && pair_vector(b, s_img, p.arith, q, qimg, pj, wrap, rx, ry, rz))
                {
                    rsq = dot3(rx, ry, rz);
                    ok = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                }
            }
            const unsigned m = __ballot_sync(FULL, ok);
            if (MODE == MODE_EMIT)
            {
                if (ok)
                {
                    const uint32_t e = found + __popc(m & ((1u << lane) - 1u));
                    if (e < EMIT_CAP)
                    {
                        const float d = __fsqrt_rn(rsq);
                        s_stage[warp].key[e] = order_key(by_distance, j, d);
                        s_stage[warp].val[e] = make_float4(rx, ry, rz, d);
                        s_stage[warp].slot[e] = static_cast<unsigned short>(e);
                    }
                }
            }
            else if (MODE == MODE_HIST)
            {
                if (ok)
                {
                    const float d = __fsqrt_rn(rsq);
                    if (!(d < h.h_min || d >= h.h_max))
                    {
                        uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                        if (bin == h.bins)
                        {
                            bin = h.bins - 1;
                        }
                        if (smem_hist)
                        {
                            atomicAdd(&my_hist[bin], 1u);
                        }
                        else
                        {
                            atomicAdd(&hist[bin], 1ull);
                        }
                    }
                }
            }
            found += __popc(m);
        }
        if (MODE == MODE_COUNT)
        {
            if (lane == 0)
            {
                counts[qi] = found;
            }
        }
        else if (MODE == MODE_EMIT)
        {
            __syncwarp();
            const int n = static_cast<int>(found);
            if (n != static_cast<int>(counts[qi]))
            {
                if (lane == 0)
                {
                    atomicExch(err, DEV_CAPACITY);
                }
                continue;
            }
            warp_sort(s_stage[warp].key, s_stage[warp].slot, n, lane);
            const uint64_t off = offsets[qi];
            for (int e = lane; e < n; e += 32)
            {
                const unsigned long long k = s_stage[warp].key[e];
                const float4 v = s_stage[warp].val[s_stage[warp].slot[e]];
                const uint32_t jj = by_distance ? static_cast<uint32_t>(k & 0xffffffffull)
                                                : static_cast<uint32_t>(k >> 32);
                ij[off + e] = make_uint2(qi, jj);
                dist[off + e] = v.w;
                vec[3 * (off + e)] = v.x;
                vec[3 * (off + e) + 1] = v.y;
                vec[3 * (off + e) + 2] = v.z;
            }
            __syncwarp();
        }
    }
    if (MODE == MODE_HIST && smem_hist)
    {
        __syncthreads();
        for (int bin = threadIdx.x; bin < static_cast<int>(h.bins); bin += blockDim.x)
        {
            unsigned long long s = 0;
            for (int c = 0; c < HIST_COPIES; ++c)
            {
                s += s_hist[c * HIST_SMEM_BINS + bin];
            }
            if (s != 0)
            {
                atomicAdd(&hist[bin], s);
            }
        }
    }
}

// Block-wide sort of one query's bonds in place in the output arrays by their
// order key: a bitonic network in its all-ascending form (each merge opens by
// comparing element e with its mirror in the block), which sorts any n when the
// missing elements past n are taken as +infinity and their comparisons skipped.
__device__ void block_sort_bonds(uint2* ij, float* dist, float* vec, uint32_t n, int by_distance)
{
    uint32_t np = 1;
    while (np < n)
    {
        np <<= 1;
    }
    auto cswap = [&](uint32_t e, uint32_t pe) {
        const uint2 a = ij[e], c = ij[pe];
        const float da = dist[e], dc = dist[pe];
        if (order_key(by_distance, a.y, da) > order_key(by_distance, c.y, dc))
        {
            ij[e] = c;
            ij[pe] = a;
            dist[e] = dc;
            dist[pe] = da;
            for (int x = 0; x < 3; ++x)
            {
                const float t = vec[3 * static_cast<size_t>(e) + x];
                vec[3 * static_cast<size_t>(e) + x] = vec[3 * static_cast<size_t>(pe) + x];
                vec[3 * static_cast<size_t>(pe) + x] = t;
            }
        }
    };
    for (uint32_t k = 2; k <= np; k <<= 1)
    {
        for (uint32_t e = threadIdx.x; e < n; e += blockDim.x)
        {
            const uint32_t pe = e ^ (k - 1);
            if ((e & (k >> 1)) == 0 && pe < n)
            {
                cswap(e, pe);
            }
        }
        __syncthreads();
        for (uint32_t j = k >> 2; j > 0; j >>= 1)
        {
            for (uint32_t e = threadIdx.x; e < n; e += blockDim.x)
            {
                const uint32_t pe = e ^ j;
                if (pe > e && pe < n)
                {
                    cswap(e, pe);
                }
            }
            __syncthreads();
        }
    }
}

// Block-per-query emit for queries with more than EMIT_CAP bonds: up to HEAVY_CAP
// are staged and sorted in shared memory; a query with more writes its bonds
// unsorted into its output rows and sorts them there.
__global__ void __launch_bounds__(256)
    k_ball_emit_heavy(DevBox b, DevGrid g, const float4* __restrict__ qpos, const uint32_t* __restrict__ qidx,
                      BallParams p, const uint32_t* __restrict__ counts, const uint64_t* __restrict__ offsets,
                      int by_distance, const uint32_t* __restrict__ list, uint2* __restrict__ ij,
                      float* __restrict__ dist, float* __restrict__ vec, int* err)
{
    extern __shared__ unsigned char smem[];
    unsigned long long* key = reinterpret_cast<unsigned long long*>(smem);
    float4* val = reinterpret_cast<float4*>(key + HEAVY_CAP);
    unsigned short* slot = reinterpret_cast<unsigned short*>(val + HEAVY_CAP);
    __shared__ float s_img[27][3];
    __shared__ unsigned int s_found;
    for (int t = threadIdx.x; t < 81; t += blockDim.x)
    {
        s_img[t / 3][t % 3] = b.img[t / 3][t % 3];
    }
    const uint32_t t = list[blockIdx.x];
    const float4 q = qpos[t];
    const uint32_t qi = qidx[t];
    const uint32_t n = counts[qi];
    if (threadIdx.x == 0)
    {
        s_found = 0;
    }
    __syncthreads();
    const bool huge = n > HEAVY_CAP;
    const uint64_t off = offsets[qi];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    int cx, cy, cz, qimg;
    query_cell(b, g, q, cx, cy, cz, qimg);
    const Stencil st = build_stencil(b, g, cx, cy, cz, p.arith, lane);
    for (uint32_t base = static_cast<uint32_t>(warp) * 32; base < st.total; base += 32 * nwarps)
    {
        const uint32_t tt = base + lane;
        uint32_t sl;
        int wrap;
        locate(st, tt < st.total ? tt : st.total - 1, sl, wrap);
        if (tt < st.total)
        {
            const float4 pj = g.cpos[sl];
            const uint32_t j = g.cidx[sl];
            float rx, ry, rz;
            if (!(p.exclude_ii && j == qi) && pair_vector(b, s_img, p.arith, q, qimg, pj, wrap, rx, ry, rz))
            {
                const float rsq = dot3(rx, ry, rz);
                if (rsq < p.r_max_sq && rsq >= p.r_min_sq)
                {
                    const uint32_t e = atomicAdd(&s_found, 1u);
                    const float d = __fsqrt_rn(rsq);
                    if (huge)
                    {
                        if (e < n)
                        {
                            ij[off + e] = make_uint2(qi, j);
                            dist[off + e] = d;
                            vec[3 * (off + e)] = rx;
                            vec[3 * (off + e) + 1] = ry;
                            vec[3 * (off + e) + 2] = rz;
                        }
                    }
                    else if (e < HEAVY_CAP)
                    {
                        key[e] = order_key(by_distance, j, d);
                        val[e] = make_float4(rx, ry, rz, d);
                        slot[e] = static_cast<unsigned short>(e);
                    }
                }
            }
        }
    }
    __syncthreads();
    if (s_found != n)
    {
        if (threadIdx.x == 0)
        {
            atomicExch(err, DEV_CAPACITY);
        }
        return;
    }
    if (huge)
    {
        block_sort_bonds(ij + off, dist + off, vec + 3 * off, n, by_distance);
        return;
    }
    int np = 1;
    while (np < static_cast<int>(n))
    {
        np <<= 1;
    }
    for (int e = static_cast<int>(n) + threadIdx.x; e < np; e += blockDim.x)
    {
        key[e] = ~0ull;
        slot[e] = 0;
    }
    __syncthreads();
    for (int k = 2; k <= np; k <<= 1)
    {
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int e = threadIdx.x; e < np; e += blockDim.x)
            {
                const int pe = e ^ j;
                if (pe > e)
                {
                    const bool up = (e & k) == 0;
                    const unsigned long long a = key[e];
                    const unsigned long long c = key[pe];
                    if ((a > c) == up)
                    {
                        key[e] = c;
                        key[pe] = a;
                        const unsigned short tmp = slot[e];
                        slot[e] = slot[pe];
                        slot[pe] = tmp;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int e = threadIdx.x; e < static_cast<int>(n); e += blockDim.x)
    {
        const unsigned long long k = key[e];
        const float4 v = val[slot[e]];
        const uint32_t jj = by_distance ? static_cast<uint32_t>(k & 0xffffffffull) : static_cast<uint32_t>(k >> 32);
        ij[off + e] = make_uint2(qi, jj);
        dist[off + e] = v.w;
        vec[3 * (off + e)] = v.x;
        vec[3 * (off + e) + 1] = v.y;
        vec[3 * (off + e) + 2] = v.z;
    }
}

__global__ void k_hist_distances(const float* __restrict__ dist, uint64_t nb, HistParams h,
                                 unsigned long long* __restrict__ hist)
{
    // HIST_COPIES privatised copies of h.bins counters (dynamic shared memory sized
    // by the launch, so a few hundred bins leave room for a full wave of blocks)
    extern __shared__ unsigned int s_hist[];
    const bool smem_hist = h.bins <= HIST_SMEM_BINS;
    if (smem_hist)
    {
        for (int t = threadIdx.x; t < HIST_COPIES * static_cast<int>(h.bins); t += blockDim.x)
        {
            s_hist[t] = 0;
        }
    }
    __syncthreads();
    unsigned int* my = s_hist + ((threadIdx.x >> 5) % HIST_COPIES) * h.bins;
    auto add = [&](float d) {
        if (d < h.h_min || d >= h.h_max)
            return;
        uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
        if (bin == h.bins)
            bin = h.bins - 1;
        if (smem_hist)
            atomicAdd(&my[bin], 1u);
        else
            atomicAdd(&hist[bin], 1ull);
    };
    // 16-byte loads, two in flight per thread: scalar head up to the first
    // 16-byte boundary, float4 body, scalar tail
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    const uint64_t gtid = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
    const uint64_t mis = (reinterpret_cast<uintptr_t>(dist) >> 2) & 3u;
    const uint64_t head = mis == 0 ? 0 : (4 - mis < nb ? 4 - mis : nb);
    if (gtid < head)
        add(dist[gtid]);
    const uint64_t n4 = (nb - head) / 4;
    const float4* d4 = reinterpret_cast<const float4*>(dist + head);
    for (uint64_t e = gtid; e < n4; e += 2 * stride)
    {
        const float4 a = d4[e];
        const float4 b = e + stride < n4 ? d4[e + stride] : make_float4(-1.0f, -1.0f, -1.0f, -1.0f);
        add(a.x);
        add(a.y);
        add(a.z);
        add(a.w);
        if (e + stride < n4)
        {
            add(b.x);
            add(b.y);
            add(b.z);
            add(b.w);
        }
    }
    for (uint64_t e = head + 4 * n4 + gtid; e < nb; e += stride)
        add(dist[e]);
    if (smem_hist)
    {
        __syncthreads();
        for (int bin = threadIdx.x; bin < static_cast<int>(h.bins); bin += blockDim.x)
        {
            unsigned long long s = 0;
            for (int c = 0; c < HIST_COPIES; ++c)
            {
                s += s_hist[c * h.bins + bin];
            }
            if (s != 0)
            {
                atomicAdd(&hist[bin], s);
            }
        }
    }
}

int query_blocks(uint32_t nq)
{
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t want = (nq + QWARPS - 1) / QWARPS;
    const uint32_t cap = static_cast<uint32_t>(sms) * 16;
    return static_cast<int>(want < cap ? (want < 1 ? 1 : want) : cap);
}

} // namespace

void launch_ball_count(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                       const BallParams& p, uint32_t* counts, cudaStream_t s, const uint32_t* list)
{
    if (p.nq == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_ball<MODE_COUNT>", s);
        k_ball<MODE_COUNT><<<query_blocks(p.nq), QWARPS * 32, 0, s>>>(box, g, qpos, qidx, p, counts, nullptr, 0, nullptr,
                                                                       nullptr, nullptr, nullptr, nullptr, nullptr,
                                                                       HistParams {}, nullptr, list);
    }
}

void launch_ball_emit(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                      const BallParams& p, const uint32_t* counts, const uint64_t* offsets, int by_distance,
                      uint2* ij, float* dist, float* vec, uint32_t* heavy_list, uint32_t* heavy_count, int* err,
                      cudaStream_t s, const uint32_t* list)
{
    if (p.nq == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_ball<MODE_EMIT>", s);
        k_ball<MODE_EMIT><<<query_blocks(p.nq), QWARPS * 32, 0, s>>>(box, g, qpos, qidx, p, const_cast<uint32_t*>(counts),
                                                                      offsets, by_distance, ij, dist, vec, heavy_list,
                                                                      heavy_count, err, HistParams {}, nullptr, list);
    }
}

void launch_ball_emit_heavy(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                            const BallParams& p, const uint32_t* counts, const uint64_t* offsets, int by_distance,
                            const uint32_t* heavy_list, uint32_t n_heavy, uint2* ij, float* dist, float* vec,
                            int* err, cudaStream_t s)
{
    if (n_heavy == 0)
    {
        return;
    }
    const size_t smem = static_cast<size_t>(HEAVY_CAP) * (sizeof(unsigned long long) + sizeof(float4) + sizeof(unsigned short));
    static bool configured = false;
    if (!configured)
    {
        cudaFuncSetAttribute(k_ball_emit_heavy, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
        configured = true;
    }
    {
        ProfScope prof_("k_ball_emit_heavy", s);
        k_ball_emit_heavy<<<n_heavy, 256, smem, s>>>(box, g, qpos, qidx, p, counts, offsets, by_distance, heavy_list, ij,
                                                     dist, vec, err);
    }
}

void launch_ball_hist(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                      const BallParams& p, const HistParams& h, unsigned long long* hist, cudaStream_t s,
                      const uint32_t* list)
{
    if (p.nq == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_ball<MODE_HIST>", s);
        k_ball<MODE_HIST><<<query_blocks(p.nq), QWARPS * 32, 0, s>>>(box, g, qpos, qidx, p, nullptr, nullptr, 0, nullptr,
                                                                      nullptr, nullptr, nullptr, nullptr, nullptr, h,
                                                                      hist, list);
    }
}

void launch_hist_distances(const float* dist, uint64_t nb, const HistParams& h, unsigned long long* hist,
                           cudaStream_t s)
{
    if (nb == 0)
    {
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // one wave of resident blocks (a partial second wave would run alone at the end)
    const size_t smem = h.bins <= static_cast<uint32_t>(HIST_SMEM_BINS) ? sizeof(unsigned int) * HIST_COPIES * h.bins : 0;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hist_distances, 256, smem);
    uint64_t want = (nb + 255) / 256;
    const uint64_t cap = static_cast<uint64_t>(sms) * static_cast<uint64_t>(per_sm > 0 ? per_sm : 1);
    {
        ProfScope prof_("k_hist_distances", s);
        k_hist_distances<<<static_cast<unsigned>(want < cap ? want : cap), 256, smem, s>>>(dist, nb, h, hist);
    }
}

// CorrelationFunction::accumulate (CorrelationFunction.cc:79-96): for each bond
// (query i, point j) whose distance falls in a bin, count[bin] += 1 and
// sum[bin] += conj(values[j]) * query_values[i] in FP64, products rounded as
// std::complex<double> forms them (re = vr*qr + vi*qi, im = vr*qi - vi*qr; no
// contraction). Per-block shared sums (CF_SMEM_BINS bins or fewer) flushed with
// global atomics; the FP64 summation order differs from the reference's
// thread-local sums, as the reference's own order depends on its threads.
constexpr int CF_SMEM_BINS = 1024;

__global__ void k_cf_bonds(const uint2* __restrict__ ij, const float* __restrict__ dist, uint64_t nb,
                           const double2* __restrict__ values, const double2* __restrict__ qvalues, HistParams h,
                           double2* __restrict__ sums, unsigned long long* __restrict__ counts)
{
    __shared__ double s_re[CF_SMEM_BINS];
    __shared__ double s_im[CF_SMEM_BINS];
    __shared__ unsigned int s_cnt[CF_SMEM_BINS];
    const bool smem = h.bins <= CF_SMEM_BINS;
    if (smem)
    {
        for (uint32_t t = threadIdx.x; t < h.bins; t += blockDim.x)
        {
            s_re[t] = 0.0;
            s_im[t] = 0.0;
            s_cnt[t] = 0;
        }
    }
    __syncthreads();
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < nb; e += stride)
    {
        const float d = dist[e];
        if (d < h.h_min || d >= h.h_max)
            continue;
        uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
        if (bin == h.bins)
            bin = h.bins - 1;
        const uint2 b = ij[e];
        const double2 v = values[b.y];
        const double2 q = qvalues[b.x];
        const double re = __dadd_rn(__dmul_rn(v.x, q.x), __dmul_rn(v.y, q.y));
        const double im = __dsub_rn(__dmul_rn(v.x, q.y), __dmul_rn(v.y, q.x));
        if (smem)
        {
            atomicAdd(&s_re[bin], re);
            atomicAdd(&s_im[bin], im);
            atomicAdd(&s_cnt[bin], 1u);
        }
        else
        {
            atomicAdd(&sums[bin].x, re);
            atomicAdd(&sums[bin].y, im);
            atomicAdd(&counts[bin], 1ull);
        }
    }
    if (smem)
    {
        __syncthreads();
        for (uint32_t t = threadIdx.x; t < h.bins; t += blockDim.x)
        {
            if (s_cnt[t] != 0)
            {
                atomicAdd(&sums[t].x, s_re[t]);
                atomicAdd(&sums[t].y, s_im[t]);
                atomicAdd(&counts[t], static_cast<unsigned long long>(s_cnt[t]));
            }
        }
    }
}

void launch_cf_bonds(const uint2* ij, const float* dist, uint64_t nb, const double2* values, const double2* qvalues,
                     const HistParams& h, double2* sums, unsigned long long* counts, cudaStream_t s)
{
    if (nb == 0)
    {
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (nb + 255) / 256;
    const uint64_t cap = static_cast<uint64_t>(sms) * 4;
    {
        ProfScope prof_("k_cf_bonds", s);
        k_cf_bonds<<<static_cast<unsigned>(want < cap ? want : cap), 256, 0, s>>>(ij, dist, nb, values, qvalues, h,
                                                                                  sums, counts);
    }
}

} // namespace fg
