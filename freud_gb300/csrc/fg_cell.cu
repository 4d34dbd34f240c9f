// Ball queries, block per home cell.
//
// A block takes one cell of the query grid and stages the candidate set shared by
// all of its queries - the points of the 27 (9 in 2D) neighbouring cells, each
// with its cell wrap - in shared memory.
//
// Pair arithmetic is exact and identical to the warp-per-query kernels
// (AABBQuery.cc:93,125 / LinkCell.cc:522). In wrap arithmetic the exact
// box.wrap (three IEEE divisions) is expensive, so a prefilter on cell-shifted
// float positions classifies each (query, candidate) pair as certainly outside
// (> r_max + delta), certainly inside (< r_max - delta; count pass with r_min = 0)
// or undecided; undecided pairs go to a per-warp queue and are tested exactly 32
// at a time with full lanes. The prefilter is enabled only when every periodic
// axis has >= 3 cells and r_max + delta is below half the smallest plane distance,
// where the cell-derived image is the minimum image of every possible bond.
//
// Scan pass: each warp holds a chunk of 32 candidates in registers and sweeps
// the cell's queries, broadcast from shared memory.
//  - count (NeighborList): grid cells are stored sorted by point index, so the
//    staged candidates are <= 27 sorted runs; five levels of pairwise merges
//    (rank by binary search) give the cell's candidates in index order. The pass
//    stores that order per cell, one acceptance mask per (query, 32-candidate
//    chunk) and the bond count per query. Cells with more than CELL_CAP
//    candidates hand their queries to the warp-per-query kernels.
//  - histogram (fused RDF): no ordering; the candidate set is processed in tiles
//    of CELL_CAP, so dense cells stay on this path.
//    Before the merge, candidates farther than r_max (+ margin) from the bounds
//    of every query of the cell are dropped.
// Write pass: warp per cell, query by query; the set bits of a query's masks, in
// chunk order, are its bonds in the reference's (i, j) order
// (NeighborBond.h:80-95); each lane takes one bond of a round of 32, recomputes
// its exact vector and writes it at the query's offset + the bond's rank.
#include <algorithm>

#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int SWARPS = 8;
constexpr int STHREADS = SWARPS * 32;
constexpr int EWARPS = 8;
constexpr int ETHREADS = EWARPS * 32;
constexpr int EMIT_LIST = 512; // write pass: bonds per query listed in shared memory (more: per-round search)
// Candidate capacity of a cell's stencil (CAP) and queries per shared-memory
// batch of the scan pass: 1024 / 64 for the common case (five blocks per SM),
// 4096 / 32 for dense point sets (one block per SM).
template<int CAP> struct CellCfg
{
    static constexpr int QB = CAP <= 1024 ? 64 : 32;
    static constexpr int POS_BITS = CAP <= 1024 ? 10 : 12; // staged-position bits of a 32-bit merge key
};
constexpr int HIST_BINS_SMEM = 4096;

enum ScanMode
{
    SM_COUNT = 0,
    SM_HIST = 1,
};

struct Items
{
    uint32_t start[32];
    uint32_t off[33];
    int wrap[32];
    uint32_t total;
    uint32_t maxrun; // most points in one item's cell
};

// Shared memory of the scan kernels; arrays one mode does not use shrink to one
// element, so the count pass with CAP 1024 fits five blocks per SM.
template<int MODE, typename K, int CAP> struct ScanShared
{
    static constexpr int QB = CellCfg<CAP>::QB;
    union
    {
        struct
        {
            K a[CAP]; // merge ping-pong buffers (KeyTraits<K>)
            K b[CAP];
        } keys;
        unsigned int hist[MODE == SM_HIST ? HIST_BINS_SMEM : 1]; // privatised RDF histogram (histogram pass)
    } u;
    float3 ps[CAP];                   // prefilter position (wrap arithmetic)
    float4 pos[MODE == SM_HIST ? CAP : 1];   // candidate position (histogram pass)
    uint32_t j[CAP];                  // point index
    uint32_t slot[CAP];               // grid slot << 5 | cell wrap code
    unsigned char run[CAP];           // stencil item (sorted run) of each staged position
    unsigned char runc[MODE == SM_COUNT ? CAP : 1]; // run of each kept candidate (count pass)
    uint32_t keep[MODE == SM_COUNT ? CAP / 32 : 1];  // kept-candidate ballots per (round, warp)
    uint32_t keep_pre[MODE == SM_COUNT ? CAP / 32 + 1 : 1];
    float qbox[SWARPS][6];            // per-warp bounds of the cell's shifted queries (lo xyz, hi xyz)
    float qfin[6];                    // their union
    uint32_t mask[MODE == SM_COUNT ? QB : 1][CAP / 32]; // acceptance per (query, chunk), count pass
    float4 q[QB];
    float4 qs[QB];
    uint32_t qi[QB];
    uint32_t queue[SWARPS][64];       // undecided pairs: sorted index | query << 16
    Items it;
    float img[27][3];
};

// Exact pair vector (same arithmetic as the warp kernels). false: image outside +-1.
__device__ __forceinline__ bool exact_vec(const DevBox& b, const float (*img)[3], int arith, float4 q, int qimg,
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
    const int kx = img_ax(pimg, 0) - img_ax(qimg, 0) - (wrap % 3 - 1);
    const int ky = img_ax(pimg, 1) - img_ax(qimg, 1) - ((wrap / 3) % 3 - 1);
    const int kz = img_ax(pimg, 2) - img_ax(qimg, 2) - (wrap / 9 - 1);
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

// Approximate position shifted by integer lattice multiples (prefilter only).
__device__ __forceinline__ float3 shifted(const DevBox& b, float4 p, int sx, int sy, int sz)
{
    float3 r;
    r.x = p.x + sx * b.L[0] + sy * (b.L[1] * b.xy) + sz * (b.L[2] * b.xz);
    r.y = p.y + sy * b.L[1] + sz * (b.L[2] * b.yz);
    r.z = p.z + sz * b.L[2];
    return r;
}

// Stencil items of cell c (run by one warp): start, wrap and prefix offsets.
__device__ void cell_items(const DevBox& b, const DevGrid& g, int arith, int c, Items& it, int lane)
{
    const int cz = c / (g.dim[0] * g.dim[1]);
    const int cy = (c / g.dim[0]) % g.dim[1];
    const int cx = c % g.dim[0];
    uint32_t cnt = 0, st = 0;
    int wr = 13;
    // the ghost grid has real cells in z (3 layers in 2D) and no wrap: the 27
    // neighbours clipped to the grid (CellIterator.h:105-146)
    const int nst = (b.is2d && arith != ARITH_GHOST) ? 9 : 27;
    if (arith == ARITH_GHOST && lane < 27)
    {
        const int ux = cx + lane % 3 - 1;
        const int uy = cy + (lane / 3) % 3 - 1;
        const int uz = cz + lane / 9 - 1;
        if (ux >= 0 && uy >= 0 && uz >= 0 && ux < g.dim[0] && uy < g.dim[1] && uz < g.dim[2])
        {
            const int cell = ux + g.dim[0] * (uy + g.dim[1] * uz);
            st = g.start[cell];
            cnt = g.start[cell + 1] - st;
        }
    }
    else if (lane < nst)
    {
        const int dx = lane % 3 - 1;
        const int dy = (lane / 3) % 3 - 1;
        const int dz = b.is2d ? 0 : lane / 9 - 1;
        auto ok = [&](int d, int dim) {
            if (arith == ARITH_AABB || dim >= 3)
                return true;
            return dim == 1 ? d == 0 : d >= 0;
        };
        if (ok(dx, g.dim[0]) && ok(dy, g.dim[1]) && (b.is2d || ok(dz, g.dim[2])))
        {
            const int ux = cx + dx, uy = cy + dy, uz = cz + dz;
            const int wx = ux < 0 ? -1 : (ux >= g.dim[0] ? 1 : 0);
            const int wy = uy < 0 ? -1 : (uy >= g.dim[1] ? 1 : 0);
            const int wz = uz < 0 ? -1 : (uz >= g.dim[2] ? 1 : 0);
            const int cell = (ux - wx * g.dim[0]) + g.dim[0] * ((uy - wy * g.dim[1]) + g.dim[1] * (uz - wz * g.dim[2]));
            st = g.start[cell];
            cnt = g.start[cell + 1] - st;
            wr = (wx + 1) + 3 * (wy + 1) + 9 * (wz + 1);
        }
    }
    uint32_t incl = cnt;
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o)
            incl += v;
    }
    const uint32_t mx = __reduce_max_sync(FULL, cnt);
    it.start[lane] = st;
    it.off[lane] = incl - cnt;
    it.wrap[lane] = wr;
    if (lane == 31)
    {
        it.off[32] = incl;
        it.total = incl;
        it.maxrun = mx;
    }
}

__device__ __forceinline__ int item_of(const Items& it, uint32_t t)
{
    int s = 0;
#pragma unroll
    for (int step = 16; step >= 1; step >>= 1)
    {
        if (s + step < 32 && it.off[s + step] <= t)
            s += step;
    }
    return s;
}

// Merge keys: (point index, staged position) packed so that key order is point
// order with ties broken by position. 32-bit keys (index << PB | position, PB =
// 10 for CAP 1024, 12 for CAP 4096) when every index is below 2^(32 - PB), else
// 64-bit (index << 32 | position).
template<typename K, int PB> struct KeyTraits;
template<int PB> struct KeyTraits<unsigned int, PB>
{
    static constexpr int SHIFT = PB;
    __device__ static unsigned int make(uint32_t j, uint32_t pos) { return (j << SHIFT) | pos; }
    __device__ static uint32_t pos(unsigned int k) { return k & ((1u << SHIFT) - 1u); }
    __device__ static uint32_t index(unsigned int k) { return k >> SHIFT; }
};
template<int PB> struct KeyTraits<unsigned long long, PB>
{
    static constexpr int SHIFT = 32;
    __device__ static unsigned long long make(uint32_t j, uint32_t pos)
    {
        return (static_cast<unsigned long long>(j) << SHIFT) | pos;
    }
    __device__ static uint32_t pos(unsigned long long k) { return static_cast<uint32_t>(k & 0xffffffffull); }
    __device__ static uint32_t index(unsigned long long k) { return static_cast<uint32_t>(k >> SHIFT); }
};

// Number of keys in src[lo, hi) smaller than key (keys are distinct).
template<typename K>
__device__ __forceinline__ uint32_t rank_in(const K* src, uint32_t lo, uint32_t hi, K key)
{
    uint32_t a = lo, z = hi;
    while (a < z)
    {
        const uint32_t m = (a + z) >> 1;
        if (src[m] < key)
            a = m + 1;
        else
            z = m;
    }
    return a - lo;
}

template<int MODE, typename K, int CAP>
__global__ void __launch_bounds__(STHREADS, MODE == SM_COUNT ? (CAP <= 1024 ? 5 : 1) : 3)
    k_cell_scan(DevBox b, DevGrid g, DevGrid qg, BallParams p, float pre_out2, float pre_in2, float cull2,
                uint32_t* __restrict__ counts, uint32_t* __restrict__ gmask, uint32_t* __restrict__ gsorted,
                uint32_t* __restrict__ gtotal, uint32_t* overflow, uint32_t* overflow_n, HistParams h,
                unsigned long long* __restrict__ hist)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using SS = ScanShared<MODE, K, CAP>;
    SS& S = *reinterpret_cast<SS*>(smem_raw);
    using KT = KeyTraits<K, CellCfg<CAP>::POS_BITS>;
    constexpr int QB = SS::QB;
    constexpr int CHUNKS = CAP / 32;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const bool use_pre = pre_out2 > 0.0f;
    const bool cull = MODE == SM_COUNT && cull2 > 0.0f;
    const bool smem_hist = MODE == SM_HIST && h.bins <= HIST_BINS_SMEM;
    uint32_t* queue = S.queue[warp];

    for (int t = tid; t < 81; t += STHREADS)
        S.img[t / 3][t % 3] = b.img[t / 3][t % 3];
    if (MODE == SM_HIST && smem_hist)
    {
        for (int t = tid; t < static_cast<int>(h.bins); t += STHREADS)
            S.u.hist[t] = 0;
    }
    __syncthreads();

    for (int c = blockIdx.x; c < qg.ncell; c += gridDim.x)
    {
        const uint32_t q0 = qg.start[c];
        const uint32_t nqc = qg.start[c + 1] - q0;
        if (nqc == 0)
            continue;
        if (cull)
        {
            // bounds of the cell's queries in cell-shifted coordinates (the prefilter's frame)
            float lo[3] = {3e30f, 3e30f, 3e30f}, hi[3] = {-3e30f, -3e30f, -3e30f};
            for (uint32_t k = tid; k < nqc; k += STHREADS)
            {
                const float4 q = qg.cpos[q0 + k];
                const int qim = __float_as_int(q.w);
                const float3 qs = shifted(b, q, -img_ax(qim, 0), -img_ax(qim, 1), -img_ax(qim, 2));
                lo[0] = fminf(lo[0], qs.x);
                lo[1] = fminf(lo[1], qs.y);
                lo[2] = fminf(lo[2], qs.z);
                hi[0] = fmaxf(hi[0], qs.x);
                hi[1] = fmaxf(hi[1], qs.y);
                hi[2] = fmaxf(hi[2], qs.z);
            }
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                for (int o = 16; o > 0; o >>= 1)
                {
                    lo[a] = fminf(lo[a], __shfl_xor_sync(FULL, lo[a], o));
                    hi[a] = fmaxf(hi[a], __shfl_xor_sync(FULL, hi[a], o));
                }
            }
            if (lane == 0)
            {
#pragma unroll
                for (int a = 0; a < 3; ++a)
                {
                    S.qbox[warp][a] = lo[a];
                    S.qbox[warp][3 + a] = hi[a];
                }
            }
        }
        if (warp == 0)
            cell_items(b, g, p.arith, c, S.it, lane);
        __syncthreads();
        uint32_t T = S.it.total;
        // the merge needs every run sorted by point index: cells above
        // SORT_CELL_MAX points are not, so their stencils overflow too
        if (MODE == SM_COUNT && (T > CAP || S.it.maxrun > static_cast<uint32_t>(SORT_CELL_MAX)))
        {
            for (uint32_t k = tid; k < nqc; k += STHREADS)
                overflow[atomicAdd(overflow_n, 1u)] = q0 + k;
            if (tid == 0)
                gtotal[c] = 0xffffffffu;
            __syncthreads();
            continue;
        }
        const uint32_t ntiles = MODE == SM_COUNT ? 1u : (T + CAP - 1) / CAP;
        for (uint32_t tile = 0; tile < ntiles; ++tile)
        {
            const uint32_t t0 = tile * CAP;
            const uint32_t TT = min(static_cast<uint32_t>(CAP), T - t0);
            // ---- stage candidates [t0, t0 + TT) ----
            if (cull)
            {
                if (tid < 6)
                {
                    float v = S.qbox[0][tid];
                    for (int w = 1; w < SWARPS; ++w)
                        v = tid < 3 ? fminf(v, S.qbox[w][tid]) : fmaxf(v, S.qbox[w][tid]);
                    S.qfin[tid] = v;
                }
                __syncthreads();
            }
            for (uint32_t base = 0; base < TT; base += STHREADS)
            {
                const uint32_t tl = base + tid;
                bool kept = false;
                if (tl < TT)
                {
                    const uint32_t t = t0 + tl;
                    const int s = item_of(S.it, t);
                    const uint32_t slot = S.it.start[s] + (t - S.it.off[s]);
                    const float4 pp = g.cpos[slot];
                    const int wr = S.it.wrap[s];
                    const uint32_t jj = g.cidx[slot];
                    S.j[tl] = jj;
                    S.slot[tl] = (slot << 5) | static_cast<uint32_t>(wr);
                    S.run[tl] = static_cast<unsigned char>(s);
                    if (MODE == SM_HIST)
                        S.pos[tl] = pp;
                    float3 sp = make_float3(0.f, 0.f, 0.f);
                    if (use_pre || cull)
                    {
                        const int pim = __float_as_int(pp.w);
                        sp = shifted(b, pp, (wr % 3 - 1) - img_ax(pim, 0), ((wr / 3) % 3 - 1) - img_ax(pim, 1),
                                     (wr / 9 - 1) - img_ax(pim, 2));
                    }
                    if (use_pre)
                        S.ps[tl] = sp;
                    if (cull)
                    {
                        // farther than r_max (+ the prefilter's margin) from the box of
                        // every query of the cell: no bond with any of them
                        const float gx = fmaxf(fmaxf(S.qfin[0] - sp.x, sp.x - S.qfin[3]), 0.f);
                        const float gy = fmaxf(fmaxf(S.qfin[1] - sp.y, sp.y - S.qfin[4]), 0.f);
                        const float gz = fmaxf(fmaxf(S.qfin[2] - sp.z, sp.z - S.qfin[5]), 0.f);
                        kept = gx * gx + gy * gy + gz * gz <= cull2;
                    }
                    else if (MODE == SM_COUNT)
                    {
                        kept = true;
                    }
                }
                if (MODE == SM_COUNT)
                {
                    const unsigned kb = __ballot_sync(FULL, kept);
                    if (lane == 0)
                        S.keep[(base / STHREADS) * SWARPS + warp] = kb;
                }
            }
            const K* order = nullptr; // sorted keys (count pass)
            if (MODE == SM_COUNT)
            {
                __syncthreads();
                // compact the kept candidates: keys (point index, staged position) and
                // their runs in staged order, so every run stays sorted
                const uint32_t nbal = (TT + 31) / 32;
                if (warp == 0)
                {
                    uint32_t carry = 0;
                    for (int w0 = 0; w0 < CHUNKS; w0 += 32)
                    {
                        const uint32_t v = w0 + lane < static_cast<int>(nbal) ? __popc(S.keep[w0 + lane]) : 0u;
                        uint32_t incl = v;
                        for (int o = 1; o < 32; o <<= 1)
                        {
                            const uint32_t u = __shfl_up_sync(FULL, incl, o);
                            if (lane >= o)
                                incl += u;
                        }
                        S.keep_pre[w0 + lane] = carry + incl - v;
                        carry += __shfl_sync(FULL, incl, 31);
                    }
                    if (lane == 0)
                        S.keep_pre[CHUNKS] = carry;
                }
                __syncthreads();
                for (uint32_t tl = tid; tl < TT; tl += STHREADS)
                {
                    const uint32_t wi = tl >> 5;
                    const uint32_t kb = S.keep[wi];
                    if ((kb >> lane) & 1u)
                    {
                        const uint32_t pos = S.keep_pre[wi] + __popc(kb & lt);
                        S.u.keys.a[pos] = KT::make(S.j[tl], tl);
                        S.runc[pos] = S.run[tl];
                    }
                }
                T = S.keep_pre[CHUNKS];
                __syncthreads();
                // run offsets among the kept candidates (runc is ascending)
                if (tid <= 32)
                {
                    uint32_t a = 0, z = T;
                    while (a < z)
                    {
                        const uint32_t m = (a + z) >> 1;
                        if (static_cast<int>(S.runc[m]) < tid)
                            a = m + 1;
                        else
                            z = m;
                    }
                    S.it.off[tid] = a;
                }
                __syncthreads();
                // merge the <= 32 sorted runs (one per stencil item) pairwise, 5 levels
                K* src = S.u.keys.a;
                K* dst = S.u.keys.b;
                for (int L = 0; L < 5; ++L)
                {
                    for (uint32_t e = tid; e < T; e += STHREADS)
                    {
                        const int r = static_cast<int>(S.runc[e]) >> L;
                        const int pr = r ^ 1;
                        const uint32_t lo_r = S.it.off[min(r << L, 32)];
                        const uint32_t lo_p = S.it.off[min(pr << L, 32)];
                        const uint32_t hi_p = S.it.off[min((pr + 1) << L, 32)];
                        const K key = src[e];
                        const uint32_t out = min(lo_r, lo_p) + (e - lo_r) + rank_in(src, lo_p, hi_p, key);
                        dst[out] = key;
                    }
                    __syncthreads();
                    K* tmp = src;
                    src = dst;
                    dst = tmp;
                }
                order = src;
                // the sorted order (grid slot << 5 | wrap) is what the write pass replays
                for (uint32_t e = tid; e < T; e += STHREADS)
                    gsorted[static_cast<size_t>(c) * CAP + e] = S.slot[KT::pos(order[e])];
                if (tid == 0)
                    gtotal[c] = T;
            }
            __syncthreads();
            const uint32_t TC = MODE == SM_COUNT ? T : TT; // candidates swept
            const uint32_t nchunks = (TC + 31) / 32;

            for (uint32_t qb0 = 0; qb0 < nqc; qb0 += QB)
            {
                const uint32_t nb = min(static_cast<uint32_t>(QB), nqc - qb0);
                for (uint32_t k = tid; k < nb; k += STHREADS)
                {
                    const float4 q = qg.cpos[q0 + qb0 + k];
                    const int qim = __float_as_int(q.w);
                    S.q[k] = q;
                    S.qi[k] = qg.cidx[q0 + qb0 + k];
                    const float3 qs = use_pre ? shifted(b, q, -img_ax(qim, 0), -img_ax(qim, 1), -img_ax(qim, 2))
                                              : make_float3(0.f, 0.f, 0.f);
                    S.qs[k] = make_float4(qs.x, qs.y, qs.z, 0.f);
                }
                __syncthreads();
                uint32_t qn = 0;

                // exact test of the first n queued (candidate, query) pairs
                auto process = [&](uint32_t n) {
                    bool acc = false;
                    float rsq = 0.f;
                    uint32_t e = 0, qq = 0;
                    if (lane < static_cast<int>(n))
                    {
                        const uint32_t ent = queue[lane];
                        e = ent & 0xffffu;
                        qq = ent >> 16;
                        const uint32_t t = MODE == SM_COUNT ? KT::pos(order[e]) : e;
                        const float4 q = S.q[qq];
                        const uint32_t sl = S.slot[t];
                        const float4 pp = MODE == SM_HIST ? S.pos[t] : g.cpos[sl >> 5];
                        float rx, ry, rz;
                        if (exact_vec(b, S.img, p.arith, q, __float_as_int(q.w), pp, static_cast<int>(sl & 31u), rx, ry,
                                      rz))
                        {
                            rsq = dot3(rx, ry, rz);
                            acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                        }
                    }
                    if (acc)
                    {
                        if (MODE == SM_COUNT)
                        {
                            atomicOr(&S.mask[qq][e >> 5], 1u << (e & 31u));
                        }
                        else
                        {
                            const float d = __fsqrt_rn(rsq);
                            if (!(d < h.h_min || d >= h.h_max))
                            {
                                uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                                if (bin == h.bins)
                                    bin = h.bins - 1;
                                if (smem_hist)
                                    atomicAdd(&S.u.hist[bin], 1u);
                                else
                                    atomicAdd(&hist[bin], 1ull);
                            }
                        }
                    }
                };

                for (uint32_t ch = warp; ch < nchunks; ch += SWARPS)
                {
                    const uint32_t e = ch * 32 + lane;
                    const bool live = e < TC;
                    const uint32_t t = (MODE == SM_COUNT && live) ? KT::pos(order[e]) : e;
                    float3 ps = make_float3(3e30f, 3e30f, 3e30f);
                    uint32_t jj = 0xffffffffu;
                    if (live)
                    {
                        jj = S.j[t];
                        if (use_pre)
                            ps = S.ps[t];
                    }
                    // queue the undecided pairs of one query (warp-uniform nm != 0)
                    auto append = [&](bool need, unsigned nm, uint32_t qq) {
                        if (need)
                            queue[qn + __popc(nm & lt)] = e | (qq << 16);
                        qn += __popc(nm);
                        __syncwarp();
                        if (qn >= 32)
                        {
                            process(32);
                            const uint32_t rest = qn - 32;
                            uint32_t v = 0;
                            if (lane < static_cast<int>(rest))
                                v = queue[32 + lane];
                            __syncwarp();
                            if (lane < static_cast<int>(rest))
                                queue[lane] = v;
                            __syncwarp();
                            qn = rest;
                        }
                    };
                    uint32_t qq = 0;
                    if (p.arith == ARITH_GHOST)
                    {
                        // stored copies: r = g - q, every pair tested in place
                        float4 pp = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (live)
                            pp = MODE == SM_HIST ? S.pos[t] : g.cpos[S.slot[t] >> 5];
                        for (; qq < nb; ++qq)
                        {
                            const float4 q = S.q[qq];
                            const bool ok = live && (MODE == SM_COUNT || !(p.exclude_ii && jj == S.qi[qq]));
                            bool acc = false;
                            float rsq = 0.f;
                            if (ok)
                            {
                                rsq = dot3(__fsub_rn(pp.x, q.x), __fsub_rn(pp.y, q.y), __fsub_rn(pp.z, q.z));
                                acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                            }
                            if (MODE == SM_COUNT)
                            {
                                const unsigned am = __ballot_sync(FULL, acc);
                                if (lane == 0)
                                    S.mask[qq][ch] = am;
                            }
                            else if (acc)
                            {
                                const float d = __fsqrt_rn(rsq);
                                if (!(d < h.h_min || d >= h.h_max))
                                {
                                    uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                                    if (bin == h.bins)
                                        bin = h.bins - 1;
                                    if (smem_hist)
                                        atomicAdd(&S.u.hist[bin], 1u);
                                    else
                                        atomicAdd(&hist[bin], 1ull);
                                }
                            }
                        }
                    }
                    if (p.arith == ARITH_AABB)
                    {
                        // AABB arithmetic is cheap, so every pair is tested exactly in place:
                        // r = p_j - (q + image_k) with k = n_j - wrap - n_q. For queries inside
                        // the box (n_q = 0) the image depends on the candidate only.
                        float4 pp = make_float4(0.f, 0.f, 0.f, 0.f);
                        int wr = 13, kx = 0, ky = 0, kz = 0;
                        if (live)
                        {
                            const uint32_t sl = S.slot[t];
                            pp = MODE == SM_HIST ? S.pos[t] : g.cpos[sl >> 5];
                            wr = static_cast<int>(sl & 31u);
                            const int pim = __float_as_int(pp.w);
                            kx = img_ax(pim, 0) - (wr % 3 - 1);
                            ky = img_ax(pim, 1) - ((wr / 3) % 3 - 1);
                            kz = img_ax(pim, 2) - (wr / 9 - 1);
                        }
                        const bool inimg = live && kx >= -1 && kx <= 1 && ky >= -1 && ky <= 1 && kz >= -1 && kz <= 1;
                        float ix = 0.f, iy = 0.f, iz = 0.f;
                        if (inimg)
                        {
                            const float* iv = S.img[(kx + 1) * 9 + (ky + 1) * 3 + (kz + 1)];
                            ix = iv[0];
                            iy = iv[1];
                            iz = iv[2];
                        }
                        for (; qq < nb; ++qq)
                        {
                            const float4 q = S.q[qq];
                            const int qimg = __float_as_int(q.w);
                            const bool ok = MODE == SM_COUNT || !(p.exclude_ii && jj == S.qi[qq]);
                            bool acc = false;
                            float rsq = 0.f;
                            if (qimg == 0)
                            {
                                if (inimg && ok)
                                {
                                    const float rx = __fsub_rn(pp.x, __fadd_rn(q.x, ix));
                                    const float ry = __fsub_rn(pp.y, __fadd_rn(q.y, iy));
                                    const float rz = __fsub_rn(pp.z, __fadd_rn(q.z, iz));
                                    rsq = dot3(rx, ry, rz);
                                    acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                                }
                            }
                            else if (live && ok)
                            {
                                float rx, ry, rz;
                                if (exact_vec(b, S.img, p.arith, q, qimg, pp, wr, rx, ry, rz))
                                {
                                    rsq = dot3(rx, ry, rz);
                                    acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                                }
                            }
                            if (MODE == SM_COUNT)
                            {
                                const unsigned am = __ballot_sync(FULL, acc);
                                if (lane == 0)
                                    S.mask[qq][ch] = am;
                            }
                            else if (acc)
                            {
                                const float d = __fsqrt_rn(rsq);
                                if (!(d < h.h_min || d >= h.h_max))
                                {
                                    uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                                    if (bin == h.bins)
                                        bin = h.bins - 1;
                                    if (smem_hist)
                                        atomicAdd(&S.u.hist[bin], 1u);
                                    else
                                        atomicAdd(&hist[bin], 1ull);
                                }
                            }
                        }
                    }
                    if (use_pre)
                    {
                        // four queries per step: independent distance tests and ballots
                        for (; qq + 4 <= nb; qq += 4)
                        {
                            bool ok[4], in[4], nd[4];
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                            {
                                const float4 qs = S.qs[qq + k];
                                const float dx = ps.x - qs.x, dy = ps.y - qs.y, dz = ps.z - qs.z;
                                const float d2 = dx * dx + dy * dy + dz * dz;
                                ok[k] = live && (MODE == SM_COUNT || !(p.exclude_ii && jj == S.qi[qq + k]));
                                in[k] = MODE == SM_COUNT && ok[k] && d2 < pre_in2;
                                nd[k] = ok[k] && !in[k] && d2 <= pre_out2;
                            }
                            if (MODE == SM_COUNT)
                            {
                                unsigned im[4];
#pragma unroll
                                for (int k = 0; k < 4; ++k)
                                    im[k] = __ballot_sync(FULL, in[k]);
                                if (lane < 4)
                                    S.mask[qq + lane][ch] = lane == 0 ? im[0] : (lane == 1 ? im[1] : (lane == 2 ? im[2] : im[3]));
                            }
                            // undecided pairs are rare (a shell of width 2 delta): one vote
                            // for the four queries, ballots only when there are some
                            if (__any_sync(FULL, nd[0] || nd[1] || nd[2] || nd[3]))
                            {
#pragma unroll
                                for (int k = 0; k < 4; ++k)
                                {
                                    const unsigned nm = __ballot_sync(FULL, nd[k]);
                                    if (nm != 0)
                                        append(nd[k], nm, qq + k);
                                }
                            }
                        }
                    }
                    for (; qq < nb; ++qq)
                    {
                        // count pass: self bonds are removed per query after the sweep
                        const bool ok = live && (MODE == SM_COUNT || !(p.exclude_ii && jj == S.qi[qq]));
                        bool need = ok;
                        bool inside = false;
                        if (use_pre)
                        {
                            const float4 qs = S.qs[qq];
                            const float dx = ps.x - qs.x, dy = ps.y - qs.y, dz = ps.z - qs.z;
                            const float d2 = dx * dx + dy * dy + dz * dz;
                            inside = MODE == SM_COUNT && ok && d2 < pre_in2;
                            need = ok && !inside && d2 <= pre_out2;
                        }
                        if (MODE == SM_COUNT)
                        {
                            const unsigned im = __ballot_sync(FULL, inside);
                            if (lane == 0)
                                S.mask[qq][ch] = im;
                        }
                        const unsigned nm = __ballot_sync(FULL, need);
                        if (nm != 0)
                            append(need, nm, qq);
                    }
                    if (MODE == SM_COUNT && qn > 0)
                    {
                        // flush before the chunk's masks can be read by another warp
                        process(qn);
                        __syncwarp();
                        qn = 0;
                    }
                }
                if (qn > 0)
                {
                    process(qn);
                    __syncwarp();
                }
                __syncthreads();
                if (MODE == SM_COUNT)
                {
                    if (p.exclude_ii)
                    {
                        // drop the bonds whose point index equals the query index
                        // (NeighborQuery exclude_ii); equal indices are adjacent in the sorted keys
                        for (uint32_t k = tid; k < nb; k += STHREADS)
                        {
                            const K lo_key = KT::make(S.qi[k], 0u);
                            uint32_t e = rank_in(order, 0, T, lo_key);
                            while (e < T && KT::index(order[e]) == S.qi[k])
                            {
                                atomicAnd(&S.mask[k][e >> 5], ~(1u << (e & 31u)));
                                ++e;
                            }
                        }
                        __syncthreads();
                    }
                    // masks and counts of this query batch: warp per query, lanes over chunks
                    for (uint32_t k = warp; k < nb; k += SWARPS)
                    {
                        uint32_t cnt = 0;
                        for (int ch = lane; ch < CHUNKS; ch += 32)
                        {
                            const uint32_t m = ch < static_cast<int>(nchunks) ? S.mask[k][ch] : 0u;
                            gmask[static_cast<size_t>(q0 + qb0 + k) * CHUNKS + ch] = m;
                            cnt += __popc(m);
                        }
                        for (int o = 16; o > 0; o >>= 1)
                            cnt += __shfl_xor_sync(FULL, cnt, o);
                        if (lane == 0)
                            counts[S.qi[k]] = cnt;
                    }
                    __syncthreads();
                }
            }
        }
    }
    if (MODE == SM_HIST && smem_hist)
    {
        __syncthreads();
        for (int bin = tid; bin < static_cast<int>(h.bins); bin += STHREADS)
        {
            if (S.u.hist[bin] != 0)
                atomicAdd(&hist[bin], static_cast<unsigned long long>(S.u.hist[bin]));
        }
    }
}

// ---------------------------------------------------------------------------
// NeighborList count pass with lanes over queries (wrap arithmetic under the
// cell-shift prefilter). A block of NLW warps takes one home cell:
//  1. bounds of the cell's queries in cell-shifted coordinates;
//  2. the stencil's candidates, a warp per stencil item (cell), culled against
//     those bounds: a first sweep counts the kept candidates of each item, a
//     second gives each its compact position t (items keep their order, so the
//     kept candidates still form one index-sorted run per item) with the key
//     (point index, t) and slot << 5 | wrap;
//  3. the runs merged into point-index order by merge path: a thread owns a
//     fixed range of output positions, finds where it starts in the two runs
//     being merged by a binary search on the cross diagonal and merges it
//     sequentially (about T / threads + log T steps per thread and level); the
//     sorted candidates' prefilter positions and indices are then gathered;
//  4. the sweep: lane = query, candidates broadcast from shared memory in index
//     order, one 32-bit word of acceptance bits per 32 candidates kept in
//     registers, so no per-pair ballot. Pairs inside r_max - delta are accepted,
//     pairs beyond r_max + delta rejected and the few in between collected in a
//     second word and tested exactly (box.wrap) once per 32 candidates. The
//     pair of a query with its own index (exclude_ii) is found once per query by
//     a binary search in the sorted keys (each point appears once in a stencil
//     of distinct cells) and its bit cleared.
// The outputs are those of the count mode of k_cell_scan: counts[query index],
// gmask rows (sorted query position x CELL_CHUNKS words), gsorted[cell][e] =
// slot << 5 | wrap of sorted candidate e, gtotal[cell]; cells over the capacity
// hand their queries to the warp-per-query kernels through overflow.
constexpr int NLW = 4; // warps per block
constexpr int NLT = NLW * 32;

// Prefilter position of a candidate: p moved into the box by its integer image
// and by the lattice shift w of its cell's wrap (an approximation within the
// prefilter's margin; both staging sweeps use it identically).
__device__ __forceinline__ float3 nl_shifted(const DevBox& b, float4 p, const float* w)
{
    const int pim = __float_as_int(p.w);
    if (pim != 0)
    {
        const float3 n = shifted(b, make_float4(0.f, 0.f, 0.f, 0.f), -img_ax(pim, 0), -img_ax(pim, 1),
                                 -img_ax(pim, 2));
        p.x += n.x;
        p.y += n.y;
        p.z += n.z;
    }
    return make_float3(p.x + w[0], p.y + w[1], p.z + w[2]);
}

// The kept flags of the staging sweeps live where the sorted candidates go later
// (rec is written after the merge), and the per-query bond counts in the merge
// buffer the merge leaves free: 29 KB per block, seven blocks per SM.
template<typename K> struct NlShared
{
    K ka[CELL_CAP];
    K kb[CELL_CAP];
    uint32_t sw[CELL_CAP];   // slot << 5 | wrap, by compact position
    union
    {
        float4 rec[CELL_CAP];                // sorted candidates: prefilter position, point index (bits)
        uint32_t kw[27][SORT_CELL_MAX / 32]; // staging: kept flags of each item's candidates
    };
    uint32_t kc[32];         // kept candidates per item
    uint32_t ro[33];         // kept-run offsets (runs past the items are empty)
    float wsh[32][3];        // lattice shift of each cell wrap code (0 .. 26)
    float qb[NLW][6];
    Items it;
    int over;
};

// One merge-path level: runs are groups of G consecutive items (offsets ro,
// ro[32] = total); pairs of groups (2k, 2k + 1) are merged from src into dst.
// This thread writes outputs [e0, e1). The output loop has no branches: the
// taken side's next key is reloaded through a selected index (clamped into the
// array; a key read past a run's end is never selected).
template<typename K>
__device__ __forceinline__ void nl_merge_level(const K* __restrict__ src, K* __restrict__ dst,
                                               const uint32_t* __restrict__ ro, int G, uint32_t e0, uint32_t e1)
{
    if (e0 >= e1)
        return;
    const int npairs = 16 / G;
    // last pair starting at or before e0 (it contains e0: the next one starts after it)
    int k = 0;
#pragma unroll
    for (int step = 8; step >= 1; step >>= 1)
    {
        if (k + step < npairs && ro[2 * (k + step) * G] <= e0)
            k += step;
    }
    uint32_t e = e0;
    while (e < e1)
    {
        const uint32_t a0 = ro[2 * k * G];
        const uint32_t a1 = ro[(2 * k + 1) * G];
        const uint32_t b1 = ro[(2 * k + 2) * G];
        const uint32_t na = a1 - a0, nb = b1 - a1;
        const uint32_t d = e - a0;
        // i = number of A keys among the first d merged keys (keys are distinct)
        uint32_t lo = d > nb ? d - nb : 0u, hi = min(d, na);
        while (lo < hi)
        {
            const uint32_t mid = (lo + hi) >> 1;
            const bool before = src[a0 + mid] < src[a1 + d - 1 - mid];
            lo = before ? mid + 1 : lo;
            hi = before ? hi : mid;
        }
        uint32_t i = lo, j = d - lo;
        K va = src[min(a0 + i, static_cast<uint32_t>(CELL_CAP - 1))];
        K vb = src[min(a1 + j, static_cast<uint32_t>(CELL_CAP - 1))];
        const uint32_t stop = min(e1, b1);
        for (; e < stop; ++e)
        {
            const bool ta = i < na && (j >= nb || va < vb);
            dst[e] = ta ? va : vb;
            i += ta ? 1u : 0u;
            j += ta ? 0u : 1u;
            const K nv = src[min(ta ? a0 + i : a1 + j, static_cast<uint32_t>(CELL_CAP - 1))];
            va = ta ? nv : va;
            vb = ta ? vb : nv;
        }
        ++k;
    }
}

template<typename K>
__global__ void __launch_bounds__(NLT, 6)
    k_nl_count(DevBox b, DevGrid g, DevGrid qg, BallParams p, float pre_out2, float pre_in2, float cull2,
               uint32_t* __restrict__ counts, uint32_t* __restrict__ gmask, uint32_t* __restrict__ gsorted,
               uint32_t* __restrict__ gtotal, uint32_t* __restrict__ overflow, uint32_t* __restrict__ overflow_n)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    NlShared<K>& S = *reinterpret_cast<NlShared<K>*>(smem_raw);
    using KT = KeyTraits<K, 10>;
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int nitems = b.is2d ? 9 : 27;

    for (int c = blockIdx.x; c < qg.ncell; c += gridDim.x)
    {
        const uint32_t q0 = qg.start[c];
        const uint32_t nqc = qg.start[c + 1] - q0;
        if (nqc == 0)
            continue;
        // ---- 1. bounds of the cell's queries (cell-shifted) and the stencil items
        {
            float lo[3] = {3e30f, 3e30f, 3e30f}, hi[3] = {-3e30f, -3e30f, -3e30f};
            for (uint32_t k = tid; k < nqc; k += NLT)
            {
                const float4 q = qg.cpos[q0 + k];
                const int qim = __float_as_int(q.w);
                const float3 qs = shifted(b, q, -img_ax(qim, 0), -img_ax(qim, 1), -img_ax(qim, 2));
                lo[0] = fminf(lo[0], qs.x);
                lo[1] = fminf(lo[1], qs.y);
                lo[2] = fminf(lo[2], qs.z);
                hi[0] = fmaxf(hi[0], qs.x);
                hi[1] = fmaxf(hi[1], qs.y);
                hi[2] = fmaxf(hi[2], qs.z);
            }
#pragma unroll
            for (int a = 0; a < 3; ++a)
            {
                for (int o = 16; o > 0; o >>= 1)
                {
                    lo[a] = fminf(lo[a], __shfl_xor_sync(FULL, lo[a], o));
                    hi[a] = fmaxf(hi[a], __shfl_xor_sync(FULL, hi[a], o));
                }
            }
            if (lane == 0)
            {
#pragma unroll
                for (int a = 0; a < 3; ++a)
                {
                    S.qb[warp][a] = lo[a];
                    S.qb[warp][3 + a] = hi[a];
                }
            }
            if (warp == 0)
            {
                cell_items(b, g, ARITH_WRAP, c, S.it, lane);
                const float3 w = shifted(b, make_float4(0.f, 0.f, 0.f, 0.f), lane % 3 - 1, (lane / 3) % 3 - 1,
                                         lane / 9 - 1);
                S.wsh[lane][0] = w.x;
                S.wsh[lane][1] = w.y;
                S.wsh[lane][2] = w.z;
            }
        }
        __syncthreads();
        float qf[6];
#pragma unroll
        for (int a = 0; a < 6; ++a)
        {
            float v = S.qb[0][a];
            for (int w = 1; w < NLW; ++w)
                v = a < 3 ? fminf(v, S.qb[w][a]) : fmaxf(v, S.qb[w][a]);
            qf[a] = v;
        }
        const bool too_big = S.it.maxrun > static_cast<uint32_t>(SORT_CELL_MAX);
        // ---- 2. staging: a warp per item; kept = within the cull radius of the bounds
        auto cand = [&](int s, uint32_t k, uint32_t& slot, int& wr, float4& pp) {
            slot = S.it.start[s] + k;
            wr = S.it.wrap[s];
            pp = g.cpos[slot];
            const float3 sp = nl_shifted(b, pp, S.wsh[wr]);
            const float gx = fmaxf(fmaxf(qf[0] - sp.x, sp.x - qf[3]), 0.f);
            const float gy = fmaxf(fmaxf(qf[1] - sp.y, sp.y - qf[4]), 0.f);
            const float gz = fmaxf(fmaxf(qf[2] - sp.z, sp.z - qf[5]), 0.f);
            return gx * gx + gy * gy + gz * gz <= cull2;
        };
        if (!too_big)
        {
            for (int s = warp; s < nitems; s += NLW)
            {
                const uint32_t n_s = S.it.off[s + 1] - S.it.off[s];
                uint32_t kept = 0;
                for (uint32_t k0 = 0; k0 < n_s; k0 += 32)
                {
                    bool keep = false;
                    if (k0 + lane < n_s)
                    {
                        uint32_t slot;
                        int wr;
                        float4 pp;
                        keep = cand(s, k0 + lane, slot, wr, pp);
                    }
                    const unsigned kb = __ballot_sync(FULL, keep);
                    if (lane == 0)
                        S.kw[s][k0 >> 5] = kb;
                    kept += __popc(kb);
                }
                if (lane == 0)
                    S.kc[s] = kept;
            }
        }
        __syncthreads();
        if (warp == 0)
        {
            const uint32_t v = (!too_big && lane < nitems) ? S.kc[lane] : 0u;
            uint32_t incl = v;
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t u = __shfl_up_sync(FULL, incl, o);
                if (lane >= o)
                    incl += u;
            }
            S.ro[lane] = incl - v;
            if (lane == 31)
            {
                S.ro[32] = incl;
                S.over = too_big || incl > static_cast<uint32_t>(CELL_CAP);
            }
        }
        __syncthreads();
        if (S.over)
        {
            for (uint32_t k = tid; k < nqc; k += NLT)
                overflow[atomicAdd(overflow_n, 1u)] = q0 + k;
            if (tid == 0)
                gtotal[c] = 0xffffffffu;
            __syncthreads();
            continue;
        }
        const uint32_t T = S.ro[32];
        for (int s = warp; s < nitems; s += NLW)
        {
            const uint32_t n_s = S.it.off[s + 1] - S.it.off[s];
            uint32_t pos = S.ro[s];
            const int wr = S.it.wrap[s];
            for (uint32_t k0 = 0; k0 < n_s; k0 += 32)
            {
                const unsigned kb = S.kw[s][k0 >> 5];
                if ((kb >> lane) & 1u)
                {
                    const uint32_t slot = S.it.start[s] + k0 + static_cast<uint32_t>(lane);
                    const uint32_t t = pos + __popc(kb & lt);
                    S.ka[t] = KT::make(g.cidx[slot], t);
                    S.sw[t] = (slot << 5) | static_cast<uint32_t>(wr);
                }
                pos += __popc(kb);
            }
        }
        __syncthreads();
        // ---- 3. merge the runs into point-index order, gather the sorted candidates
        K* src = S.ka;
        K* dst = S.kb;
        {
            // every thread merges (a merge level is a barrier-bound step: the block's
            // other warps would only wait; 0.99 ms against 1.02 ms with 64 threads on
            // the 102^3 lattice, 1.09 ms with 32)
            constexpr int NLM = NLT;
            const uint32_t per = (T + NLM - 1) / NLM;
            const uint32_t e0 = tid < NLM ? min(T, per * tid) : T;
            const uint32_t e1 = tid < NLM ? min(T, e0 + per) : T;
            for (int G = 1; G < nitems; G <<= 1)
            {
                nl_merge_level(src, dst, S.ro, G, e0, e1);
                __syncthreads();
                K* tmp = src;
                src = dst;
                dst = tmp;
            }
        }
        const K* order = src;
        // bond counts of the cell's queries, in the merge buffer the merge left free
        uint32_t* cnt = reinterpret_cast<uint32_t*>(dst);
        for (uint32_t k = tid; k < nqc && k < static_cast<uint32_t>(CELL_CAP); k += NLT)
            cnt[k] = 0;
        for (uint32_t e = tid; e < T; e += NLT)
        {
            const K key = order[e];
            const uint32_t sw = S.sw[KT::pos(key)];
            gsorted[static_cast<size_t>(c) * CELL_CAP + e] = sw;
            const float4 pp = g.cpos[sw >> 5];
            const float3 sp = nl_shifted(b, pp, S.wsh[sw & 31u]);
            S.rec[e] = make_float4(sp.x, sp.y, sp.z, __uint_as_float(KT::index(key)));
        }
        if (tid == 0)
            gtotal[c] = T;
        __syncthreads();
        // ---- 4. sweep: lane = query, candidates in index order
        const uint32_t nchunks = (T + 31) / 32;
        const uint32_t ngroups = (nqc + 31) / 32;
        uint32_t cur_group = 0xffffffffu;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
        float3 qs = make_float3(3e30f, 3e30f, 3e30f);
        uint32_t self_e = 0xffffffffu; // sorted position of the query's own index
        for (uint32_t item = warp; item < ngroups * nchunks; item += NLW)
        {
            const uint32_t gq = item / nchunks;
            const uint32_t ch = item - gq * nchunks;
            const uint32_t qk = gq * 32 + lane;
            const bool live = qk < nqc;
            if (gq != cur_group)
            {
                cur_group = gq;
                qs = make_float3(3e30f, 3e30f, 3e30f);
                self_e = 0xffffffffu;
                if (live)
                {
                    q = qg.cpos[q0 + qk];
                    const uint32_t qi = qg.cidx[q0 + qk];
                    const int qim = __float_as_int(q.w);
                    qs = shifted(b, q, -img_ax(qim, 0), -img_ax(qim, 1), -img_ax(qim, 2));
                    if (p.exclude_ii)
                    {
                        // first sorted key with index >= qi
                        uint32_t lo = 0, hi = T;
                        const K kq = KT::make(qi, 0u);
                        while (lo < hi)
                        {
                            const uint32_t mid = (lo + hi) >> 1;
                            if (order[mid] < kq)
                                lo = mid + 1;
                            else
                                hi = mid;
                        }
                        if (lo < T && KT::index(order[lo]) == qi)
                            self_e = lo;
                    }
                }
            }
            const uint32_t e0 = ch * 32;
            uint32_t word = 0, und = 0;
            const float4* rc = S.rec + e0;
            if (e0 + 32 <= T)
            {
#pragma unroll
                for (int bb = 0; bb < 32; ++bb)
                {
                    const float4 r = rc[bb];
                    const float dx = r.x - qs.x, dy = r.y - qs.y, dz = r.z - qs.z;
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 < pre_in2)
                        word |= 1u << bb;
                    if (d2 <= pre_out2)
                        und |= 1u << bb;
                }
            }
            else
            {
                const int ne = static_cast<int>(T - e0);
                for (int bb = 0; bb < ne; ++bb)
                {
                    const float4 r = rc[bb];
                    const float dx = r.x - qs.x, dy = r.y - qs.y, dz = r.z - qs.z;
                    const float d2 = dx * dx + dy * dy + dz * dz;
                    if (d2 < pre_in2)
                        word |= 1u << bb;
                    if (d2 <= pre_out2)
                        und |= 1u << bb;
                }
            }
            if (self_e - e0 < 32u)
            {
                word &= ~(1u << (self_e - e0));
                und &= ~(1u << (self_e - e0));
            }
            und &= ~word;
            // pairs between the two prefilter radii: the exact test
            while (__any_sync(FULL, und != 0))
            {
                if (und != 0)
                {
                    const int bb = __ffs(und) - 1;
                    und &= und - 1u;
                    const uint32_t sw = gsorted[static_cast<size_t>(c) * CELL_CAP + e0 + bb];
                    const float4 pp = g.cpos[sw >> 5];
                    float rx, ry, rz;
                    box_wrap(b, __fsub_rn(pp.x, q.x), __fsub_rn(pp.y, q.y), __fsub_rn(pp.z, q.z), rx, ry, rz);
                    const float rsq = dot3(rx, ry, rz);
                    if (rsq < p.r_max_sq && rsq >= p.r_min_sq)
                        word |= 1u << bb;
                }
            }
            if (live)
            {
                gmask[static_cast<size_t>(q0 + qk) * CELL_CHUNKS + ch] = word;
                atomicAdd(&cnt[qk], static_cast<uint32_t>(__popc(word)));
            }
        }
        __syncthreads();
        for (uint32_t k = tid; k < nqc; k += NLT)
            counts[qg.cidx[q0 + k]] = cnt[k];
        __syncthreads();
    }
}

// Position of the k-th (from 0) set bit of w; k < popc(w).
__device__ __forceinline__ uint32_t kth_set_bit(uint32_t w, uint32_t k)
{
    uint32_t pos = 0;
#pragma unroll
    for (int half = 16; half >= 1; half >>= 1)
    {
        const uint32_t c = __popc(w & ((1u << half) - 1u));
        if (k >= c)
        {
            k -= c;
            w >>= half;
            pos += half;
        }
    }
    return pos;
}

// Write pass, warp per cell: no block barriers. A warp takes one cell and writes
// the bonds of each of its queries: each lane lists the set bits of its chunks'
// masks (one chunk per lane with CAP 1024) as candidate positions in a per-warp
// shared list at the exclusive prefix of the per-lane bond counts, so the list
// holds the query's bonds in order; lane l then writes bonds l, l + 32, ... of
// the list. A query with more than EMIT_LIST bonds instead finds bond base + l of
// each round from the prefix sums and the k-th set bit of the chunk's mask.
// Candidates are read through the cell's sorted list (gsorted) from L1/L2, where
// the cell's other queries keep them.
template<int CAP, int ARITH>
__global__ void __launch_bounds__(ETHREADS, 4)
    k_cell_emit(DevBox b, DevGrid g, DevGrid qg, BallParams p, const uint32_t* __restrict__ gmask,
                const uint32_t* __restrict__ gsorted, const uint32_t* __restrict__ gtotal,
                const uint64_t* __restrict__ offsets, uint2* __restrict__ ij, float* __restrict__ dist,
                float* __restrict__ vec, uint32_t nq_total, uint32_t per_item)
{
    // WPL mask words per lane: lane l holds chunks l*WPL .. l*WPL + WPL - 1
    constexpr int CHUNKS = CAP / 32;
    constexpr int WPL = CHUNKS / 32;
    __shared__ float img_s[27][3];
    __shared__ uint16_t blist[EWARPS][EMIT_LIST]; // a query's bonds as candidate positions
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    for (int t = tid; t < 81; t += ETHREADS)
        img_s[t / 3][t % 3] = b.img[t / 3][t % 3];
    __syncthreads();
    // work items: one cell's queries (per_item == 0, many cells), or runs of
    // per_item consecutive cell-sorted queries (few, dense cells)
    const uint32_t nwarps = gridDim.x * EWARPS;
    const uint32_t n_items = per_item == 0 ? static_cast<uint32_t>(qg.ncell) : (nq_total + per_item - 1) / per_item;
    for (uint32_t item = blockIdx.x * EWARPS + warp; item < n_items; item += nwarps)
    {
        uint32_t k0, k1;
        int c = 0;
        if (per_item == 0)
        {
            c = static_cast<int>(item);
            k0 = qg.start[c];
            k1 = qg.start[c + 1];
        }
        else
        {
            k0 = item * per_item;
            k1 = min(k0 + per_item, nq_total);
            // cell of query k0: the last cell whose start is <= k0
            int hi = qg.ncell;
            while (hi - c > 1)
            {
                const int mid = (c + hi) >> 1;
                if (qg.start[mid] <= k0)
                    c = mid;
                else
                    hi = mid;
            }
        }
        for (uint32_t q0 = k0; q0 < k1 && c < qg.ncell; ++c)
        {
            // queries [q0, q0 + nqc) of cell c within this item
            const uint32_t cend = qg.start[c + 1];
            if (cend <= q0)
                continue;
            const uint32_t nqc = min(cend, k1) - q0;
            const uint32_t qbeg = q0;
            q0 += nqc;
            const uint32_t T = gtotal[c];
            if (T > CAP)
                continue; // the cell's queries are written by the warp-per-query kernels
            const uint32_t* srt = gsorted + static_cast<size_t>(c) * CAP;
            const uint32_t nchunks = (T + 31) / 32;
            auto load_row = [&](uint32_t row, uint32_t (&w)[WPL]) {
#pragma unroll
                for (int k = 0; k < WPL; ++k)
                {
                    const uint32_t ch = static_cast<uint32_t>(lane * WPL + k);
                    w[k] = ch < nchunks ? gmask[static_cast<size_t>(row) * CHUNKS + ch] : 0u;
                }
            };
            float4 q_n = qg.cpos[qbeg];
            uint32_t qi_n = qg.cidx[qbeg];
            uint32_t mw_n[WPL];
            load_row(qbeg, mw_n);
            for (uint32_t qq = 0; qq < nqc; ++qq)
            {
                const float4 q = q_n;
                const uint32_t qi = qi_n;
                uint32_t mword[WPL];
#pragma unroll
                for (int k = 0; k < WPL; ++k)
                    mword[k] = mw_n[k];
                const int qimg = __float_as_int(q.w);
                const uint64_t out = offsets[qi];
                if (qq + 1 < nqc)
                {
                    // one-ahead prefetch of the next query (position, index, mask row)
                    q_n = qg.cpos[qbeg + qq + 1];
                    qi_n = qg.cidx[qbeg + qq + 1];
                    load_row(qbeg + qq + 1, mw_n);
                }
                uint32_t cnt = 0;
#pragma unroll
                for (int k = 0; k < WPL; ++k)
                    cnt += __popc(mword[k]);
                uint32_t incl = cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o)
                        incl += v;
                }
                const uint32_t excl = incl - cnt;
                const uint32_t total = __shfl_sync(FULL, incl, 31);
                // bond bb of the query: candidate position e (chunk * 32 + bit) in the cell's sorted list
                // store bond bb from its candidate (entry ent of the sorted list, position pp, index jj)
                auto store_bond = [&](uint32_t bb, uint32_t ent, float4 pp, uint32_t jj) {
                    float rx, ry, rz;
                    exact_vec(b, img_s, ARITH, q, qimg, pp, static_cast<int>(ent & 31u), rx, ry, rz);
                    const uint64_t o = out + bb;
                    ij[o] = make_uint2(qi, jj);
                    dist[o] = __fsqrt_rn(dot3(rx, ry, rz));
                    vec[3 * o] = rx;
                    vec[3 * o + 1] = ry;
                    vec[3 * o + 2] = rz;
                };
                auto write_bond = [&](uint32_t bb, uint32_t e) {
                    const uint32_t ent = srt[e];
                    store_bond(bb, ent, g.cpos[ent >> 5], g.cidx[ent >> 5]);
                };
                if (total <= static_cast<uint32_t>(EMIT_LIST))
                {
                    // each lane lists the set bits of its mask words at its prefix, so
                    // the list holds the bonds in chunk order, bits ascending
                    uint16_t* lst = blist[warp];
                    uint32_t k = excl;
#pragma unroll
                    for (int kw = 0; kw < WPL; ++kw)
                    {
                        uint32_t w = mword[kw];
                        const uint32_t chb = static_cast<uint32_t>(lane * WPL + kw) * 32u;
                        while (w != 0)
                        {
                            lst[k++] = static_cast<uint16_t>(chb + static_cast<uint32_t>(__ffs(w) - 1));
                            w &= w - 1u;
                        }
                    }
                    __syncwarp();
                    // one bond ahead: the next bond's candidate loads are issued before
                    // this bond's stores (the grid arrays may alias the outputs as far as
                    // the compiler knows, so it would not hoist them itself)
                    uint32_t bb = lane;
                    uint32_t ent = 0, jj = 0;
                    float4 pp = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (bb < total)
                    {
                        ent = srt[lst[bb]];
                        pp = g.cpos[ent >> 5];
                        jj = g.cidx[ent >> 5];
                    }
                    while (bb < total)
                    {
                        const uint32_t bn = bb + 32u;
                        uint32_t ent_n = 0, jj_n = 0;
                        float4 pp_n = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (bn < total)
                        {
                            ent_n = srt[lst[bn]];
                            pp_n = g.cpos[ent_n >> 5];
                            jj_n = g.cidx[ent_n >> 5];
                        }
                        store_bond(bb, ent, pp, jj);
                        bb = bn;
                        ent = ent_n;
                        pp = pp_n;
                        jj = jj_n;
                    }
                    __syncwarp();
                    continue;
                }
                for (uint32_t base = 0; base < total; base += 32)
                {
                    const uint32_t bb = base + static_cast<uint32_t>(lane);
                    // lane holding bond bb: the last lane whose exclusive prefix is <= bb
                    int ln = 0;
#pragma unroll
                    for (int step = 16; step >= 1; step >>= 1)
                    {
                        const uint32_t v = __shfl_sync(FULL, excl, ln + step);
                        if (v <= bb)
                            ln += step;
                    }
                    uint32_t k = bb - __shfl_sync(FULL, excl, ln);
                    // then the word of that lane, in chunk order
                    uint32_t w = 0, ch = 0;
                    bool found = false;
#pragma unroll
                    for (int kw = 0; kw < WPL; ++kw)
                    {
                        const uint32_t wk = __shfl_sync(FULL, mword[kw], ln);
                        const uint32_t ck = __popc(wk);
                        if (!found)
                        {
                            if (k < ck)
                            {
                                w = wk;
                                ch = static_cast<uint32_t>(ln * WPL + kw);
                                found = true;
                            }
                            else
                            {
                                k -= ck;
                            }
                        }
                    }
                    if (bb < total)
                        write_bond(bb, ch * 32u + kth_set_bit(w, k));
                }
            }
        }
    }
}

// Write pass, block per cell, the bonds of all the cell's queries in full rounds
// of 32 with no global load per bond. The block stages the cell's sorted
// candidates (position, point index) in shared memory. For each group of 32 of
// the cell's queries, warp 0 takes the exclusive prefix of the group's bond
// counts (queries whose bonds would pass the list's capacity wait for the next
// window); the warps then split each query's mask row by word ranges (lane =
// query), count their bits, and list them, in order, as candidate positions (and
// the bond's query) after the bits of the lower ranges; then every warp takes
// rounds of 32 bonds: a bond's query and candidate come from the list, and it
// writes the exact vector at the query's offset plus the bond's rank.
constexpr int WW = 4;        // warps per block
constexpr int WLIST = 4096;  // listed bonds per window

struct NlWriteShared
{
    float4 cp[CELL_CAP];      // sorted candidates: position (w = packed box image)
    uint32_t cj[CELL_CAP];    // point index
    uint8_t cw[CELL_CAP];     // cell wrap code
    uint16_t lst[WLIST];      // listed bond: candidate position | query (lane of the group) << 10
    float4 qp[32];
    uint32_t qi[32];
    unsigned long long qo[32]; // output offset of the query's bonds minus its prefix in the list
    uint32_t pre[33];
    uint32_t wcnt[WW][32];    // bits of each warp's word range, per query
    float img[27][3];
};

template<int ARITH>
__global__ void __launch_bounds__(WW * 32, 7)
    k_nl_write(DevBox b, DevGrid g, DevGrid qg, BallParams p, const uint32_t* __restrict__ gmask,
               const uint32_t* __restrict__ gsorted, const uint32_t* __restrict__ gtotal,
               const uint32_t* __restrict__ counts, const uint64_t* __restrict__ offsets, uint2* __restrict__ ij,
               float* __restrict__ dist, float* __restrict__ vec)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    NlWriteShared& S = *reinterpret_cast<NlWriteShared*>(smem_raw);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    for (int t = tid; t < 81; t += WW * 32)
        S.img[t / 3][t % 3] = b.img[t / 3][t % 3];
    for (int c = blockIdx.x; c < qg.ncell; c += gridDim.x)
    {
        const uint32_t q0 = qg.start[c];
        const uint32_t nqc = qg.start[c + 1] - q0;
        if (nqc == 0)
            continue;
        const uint32_t T = gtotal[c];
        if (T > static_cast<uint32_t>(CELL_CAP))
            continue; // the cell's queries are written by the warp-per-query kernels
        const uint32_t nchunks = (T + 31) / 32;
        __syncthreads(); // the previous cell's rounds are done with the shared arrays
        {
            // the cell's sorted candidates, four per thread at a time with every load
            // issued before any use
            constexpr int PER = 4;
            for (uint32_t e0 = static_cast<uint32_t>(tid); e0 < T; e0 += PER * WW * 32)
            {
                uint32_t ent[PER];
#pragma unroll
                for (int k = 0; k < PER; ++k)
                {
                    const uint32_t e = e0 + static_cast<uint32_t>(k * WW * 32);
                    ent[k] = e < T ? gsorted[static_cast<size_t>(c) * CELL_CAP + e] : 0u;
                }
                float4 cp[PER];
                uint32_t cj[PER];
#pragma unroll
                for (int k = 0; k < PER; ++k)
                {
                    const uint32_t e = e0 + static_cast<uint32_t>(k * WW * 32);
                    if (e < T)
                    {
                        cp[k] = g.cpos[ent[k] >> 5];
                        cj[k] = g.cidx[ent[k] >> 5];
                    }
                }
#pragma unroll
                for (int k = 0; k < PER; ++k)
                {
                    const uint32_t e = e0 + static_cast<uint32_t>(k * WW * 32);
                    if (e < T)
                    {
                        S.cp[e] = cp[k];
                        S.cj[e] = cj[k];
                        S.cw[e] = static_cast<uint8_t>(ent[k] & 31u);
                    }
                }
            }
        }
        for (uint32_t g0 = 0; g0 < nqc; g0 += 32)
        {
            const uint32_t qk = g0 + static_cast<uint32_t>(lane);
            const bool live = qk < nqc;
            uint32_t cnt = 0, qi = 0;
            const uint32_t* row = gmask + static_cast<size_t>(q0 + qk) * CELL_CHUNKS;
            if (warp == 0 && live)
            {
                qi = qg.cidx[q0 + qk];
                cnt = counts[qi];
            }
            int la = 0;
            while (la < 32)
            {
                __syncthreads(); // the previous window's rounds are done with the shared arrays
                if (warp == 0)
                {
                    if (la == 0 && live)
                    {
                        S.qp[lane] = qg.cpos[q0 + qk];
                        S.qi[lane] = qi;
                    }
                    // exclusive prefix of the counts of lanes la .. 31
                    const uint32_t cl = lane >= la ? cnt : 0u;
                    uint32_t incl = cl;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1)
                    {
                        const uint32_t v = __shfl_up_sync(FULL, incl, o);
                        if (lane >= o)
                            incl += v;
                    }
                    const uint32_t pre = incl - cl;
                    const bool in_win = lane >= la && incl <= static_cast<uint32_t>(WLIST);
                    const unsigned wm = __ballot_sync(FULL, in_win);
                    const int lb = 32 - __clz(wm); // a query never exceeds the list
                    const uint32_t total = __shfl_sync(FULL, incl, lb - 1);
                    S.pre[lane] = pre;
                    if (in_win && live)
                        S.qo[lane] = offsets[qi] - pre; // + the bond's list position (>= pre)
                    if (lane == 0)
                        S.pre[32] = (static_cast<uint32_t>(lb) << 16) | total;
                }
                __syncthreads();
                const uint32_t win = S.pre[32];
                const int lbw = static_cast<int>(win >> 16);
                // list building split by mask words: warp w takes words [w0, w1) of every
                // query of the window (lane = query), counts its bits, then lists them after
                // the bits of the lower word ranges
                const uint32_t per_w = (nchunks + WW - 1) / WW;
                const uint32_t w0 = min(nchunks, per_w * warp);
                const uint32_t w1 = min(nchunks, w0 + per_w);
                const bool lane_in = lane >= la && lane < lbw && live;
                uint32_t wv[8];
                uint32_t mine = 0;
                if (lane_in)
                {
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                    {
                        wv[t] = w0 + t < w1 ? row[w0 + t] : 0u;
                        mine += __popc(wv[t]);
                    }
                    for (uint32_t k = w0 + 8; k < w1; ++k)
                        mine += __popc(row[k]);
                }
                S.wcnt[warp][lane] = mine;
                __syncthreads();
                if (lane_in && mine > 0)
                {
                    uint32_t k = S.pre[lane];
                    for (int w2 = 0; w2 < warp; ++w2)
                        k += S.wcnt[w2][lane];
#pragma unroll
                    for (int t = 0; t < 8; ++t)
                    {
                        uint32_t w = wv[t];
                        while (w != 0)
                        {
                            S.lst[k++] = static_cast<uint16_t>(((w0 + t) * 32u + static_cast<uint32_t>(__ffs(w) - 1)) |
                                                               (static_cast<uint32_t>(lane) << 10));
                            w &= w - 1u;
                        }
                    }
                    for (uint32_t ch = w0 + 8; ch < w1; ++ch)
                    {
                        uint32_t w = row[ch];
                        while (w != 0)
                        {
                            S.lst[k++] = static_cast<uint16_t>((ch * 32u + static_cast<uint32_t>(__ffs(w) - 1)) |
                                                               (static_cast<uint32_t>(lane) << 10));
                            w &= w - 1u;
                        }
                    }
                }
                __syncthreads();
                const uint32_t total = win & 0xffffu;
#pragma unroll 1
                for (uint32_t bb = static_cast<uint32_t>(tid); bb < total; bb += WW * 32)
                {
                    const uint32_t le = S.lst[bb];
                    const int own = static_cast<int>(le >> 10);
                    const uint32_t e = le & 1023u;
                    const float4 q = S.qp[own];
                    float rx, ry, rz;
                    exact_vec(b, S.img, ARITH, q, __float_as_int(q.w), S.cp[e], static_cast<int>(S.cw[e]), rx, ry, rz);
                    const uint64_t o = S.qo[own] + bb;
                    ij[o] = make_uint2(S.qi[own], S.cj[e]);
                    dist[o] = __fsqrt_rn(dot3(rx, ry, rz));
                    vec[3 * o] = rx;
                    vec[3 * o + 1] = ry;
                    vec[3 * o + 2] = rz;
                }
                la = lbw;
            }
        }
    }
}

int sm_count_cell()
{
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

template<typename K> void configure(K kernel, size_t bytes, bool& done)
{
    if (!done)
    {
        cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
        done = true;
    }
}

} // namespace

size_t cell_smem_bytes()
{
    return sizeof(ScanShared<SM_COUNT, unsigned long long, 1024>);
}

int cell_cap_for(const DevGrid& g, uint32_t n_points, bool is2d)
{
    // mean candidates of a 27-cell (9 in 2D) stencil: below ~850 the largest of
    // ~10^5 uniformly filled stencils (mean + 4.5 sigma, Poisson) stays under 1024
    const double mean = static_cast<double>(n_points) / std::max(g.ncell, 1) * (is2d ? 9.0 : 27.0);
    return mean > 850.0 ? 4096 : 1024;
}

namespace {
template<int CAP>
void scan_count(const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p, float pre_out2,
                float pre_in2, float cull2, uint32_t* counts, uint32_t* gmask, uint32_t* gsorted, uint32_t* gtotal,
                uint32_t* overflow, uint32_t* overflow_n, cudaStream_t s, uint32_t n_points)
{
    auto go = [&](auto kernel, size_t smem, bool& done) {
        configure(kernel, smem, done);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, STHREADS, smem);
        const int want = std::max(per_sm, 1) * sm_count_cell();
        const int blocks = qg.ncell < want ? (qg.ncell < 1 ? 1 : qg.ncell) : want;
        ProfScope prof_("k_cell_scan<COUNT>", s);
        kernel<<<blocks, STHREADS, smem, s>>>(box, g, qg, p, pre_out2, pre_in2, cull2, counts, gmask, gsorted, gtotal,
                                              overflow, overflow_n, HistParams {}, nullptr);
    };
    // 32-bit merge keys while every point index fits beside the staged position
    if (n_points <= (1u << (32 - CellCfg<CAP>::POS_BITS)))
    {
        static bool done = false;
        go(k_cell_scan<SM_COUNT, unsigned int, CAP>, sizeof(ScanShared<SM_COUNT, unsigned int, CAP>), done);
    }
    else
    {
        static bool done = false;
        go(k_cell_scan<SM_COUNT, unsigned long long, CAP>, sizeof(ScanShared<SM_COUNT, unsigned long long, CAP>),
           done);
    }
}
} // namespace

void launch_cell_scan(int hist_mode, const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p,
                      float pre_out2, float pre_in2, float cull2, uint32_t* counts, uint32_t* gmask,
                      uint32_t* gsorted, uint32_t* gtotal, uint32_t* overflow, uint32_t* overflow_n,
                      const HistParams& h, unsigned long long* hist, cudaStream_t s, uint32_t n_points, int cap)
{
    if (!hist_mode)
    {
        if (cap > 1024)
            scan_count<4096>(box, g, qg, p, pre_out2, pre_in2, cull2, counts, gmask, gsorted, gtotal, overflow,
                             overflow_n, s, n_points);
        else
            scan_count<1024>(box, g, qg, p, pre_out2, pre_in2, cull2, counts, gmask, gsorted, gtotal, overflow,
                             overflow_n, s, n_points);
        return;
    }
    // one wave of resident blocks walking the cells
    const size_t smem = sizeof(ScanShared<SM_HIST, unsigned long long, 1024>);
    static bool done = false;
    configure(k_cell_scan<SM_HIST, unsigned long long, 1024>, smem, done);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cell_scan<SM_HIST, unsigned long long, 1024>, STHREADS,
                                                  smem);
    const int want = std::max(per_sm, 1) * sm_count_cell();
    const int blocks = qg.ncell < want ? (qg.ncell < 1 ? 1 : qg.ncell) : want;
    ProfScope prof_("k_cell_scan<HIST>", s);
    k_cell_scan<SM_HIST, unsigned long long, 1024><<<blocks, STHREADS, smem, s>>>(
        box, g, qg, p, pre_out2, 0.0f, 0.0f, counts, gmask, gsorted, gtotal, overflow, overflow_n, h, hist);
}

void launch_nl_count(const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p, float pre_out2,
                     float pre_in2, float cull2, uint32_t* counts, uint32_t* gmask, uint32_t* gsorted,
                     uint32_t* gtotal, uint32_t* overflow, uint32_t* overflow_n, cudaStream_t s, uint32_t n_points)
{
    auto go = [&](auto kernel, size_t smem, bool& done) {
        configure(kernel, smem, done);
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, NLT, smem);
        const int want = std::max(per_sm, 1) * sm_count_cell();
        const int blocks = qg.ncell < want ? std::max(qg.ncell, 1) : want;
        ProfScope prof_("k_nl_count", s);
        kernel<<<blocks, NLT, smem, s>>>(box, g, qg, p, pre_out2, pre_in2, cull2, counts, gmask, gsorted, gtotal,
                                         overflow, overflow_n);
    };
    // 32-bit keys (point index << 10 | compact position) below 2^22 points
    if (n_points <= (1u << 22))
    {
        static bool done = false;
        go(k_nl_count<unsigned int>, sizeof(NlShared<unsigned int>), done);
    }
    else
    {
        static bool done = false;
        go(k_nl_count<unsigned long long>, sizeof(NlShared<unsigned long long>), done);
    }
}

void launch_cell_emit(const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p,
                      const uint32_t* gmask, const uint32_t* gsorted, const uint32_t* gtotal, const uint64_t* offsets,
                      uint2* ij, float* dist, float* vec, cudaStream_t s, int cap, const uint32_t* counts)
{
    if (cap <= CELL_CAP && counts != nullptr)
    {
        // block per cell when the cells keep every resident block busy (two or more each)
        auto go_w = [&](auto kernel, bool& conf) {
            const size_t smem = sizeof(NlWriteShared);
            configure(kernel, smem, conf);
            int per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, WW * 32, smem);
            const int want = std::max(per_sm, 1) * sm_count_cell();
            if (static_cast<uint64_t>(qg.ncell) < 2ull * want)
                return false;
            ProfScope prof_("k_nl_write", s);
            kernel<<<want, WW * 32, smem, s>>>(box, g, qg, p, gmask, gsorted, gtotal, counts, offsets, ij, dist, vec);
            return true;
        };
        bool done = false;
        static bool conf_w = false, conf_g = false, conf_a = false;
        if (p.arith == ARITH_WRAP)
            done = go_w(k_nl_write<ARITH_WRAP>, conf_w);
        else if (p.arith == ARITH_GHOST)
            done = go_w(k_nl_write<ARITH_GHOST>, conf_g);
        else
            done = go_w(k_nl_write<ARITH_AABB>, conf_a);
        if (done)
            return;
    }
    auto go = [&](auto kernel) {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, ETHREADS, 0);
        const int want = std::max(per_sm, 1) * sm_count_cell();
        // a cell per work item when there are at least two cells per resident warp;
        // else runs of queries, about four per resident warp
        const uint64_t warps = static_cast<uint64_t>(want) * EWARPS;
        uint32_t per_item = 0;
        uint64_t items = static_cast<uint64_t>(std::max(qg.ncell, 1));
        if (items < 2 * warps)
        {
            per_item = std::max<uint32_t>(1, static_cast<uint32_t>(p.nq / (4 * warps)));
            items = (p.nq + per_item - 1) / per_item;
        }
        const uint64_t need = (items + EWARPS - 1) / EWARPS;
        const int blocks = need < static_cast<uint64_t>(want) ? static_cast<int>(std::max<uint64_t>(need, 1)) : want;
        ProfScope prof_("k_cell_emit", s);
        kernel<<<blocks, ETHREADS, 0, s>>>(box, g, qg, p, gmask, gsorted, gtotal, offsets, ij, dist, vec, p.nq,
                                           per_item);
    };
    // the pair arithmetic is a template parameter, so the per-bond vector has no
    // run-time branch on it
    if (cap > 1024)
    {
        if (p.arith == ARITH_WRAP)
            go(k_cell_emit<4096, ARITH_WRAP>);
        else if (p.arith == ARITH_GHOST)
            go(k_cell_emit<4096, ARITH_GHOST>);
        else
            go(k_cell_emit<4096, ARITH_AABB>);
    }
    else
    {
        if (p.arith == ARITH_WRAP)
            go(k_cell_emit<1024, ARITH_WRAP>);
        else if (p.arith == ARITH_GHOST)
            go(k_cell_emit<1024, ARITH_GHOST>);
        else
            go(k_cell_emit<1024, ARITH_AABB>);
    }
}

} // namespace fg
