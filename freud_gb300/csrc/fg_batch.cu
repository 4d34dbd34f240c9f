// Batched frames: every frame of a batch of uneven-N frames in one launch per
// stage.
//
// Grid build: one counting sort over the concatenated points, each point placed
// by its own frame's box (exact makeFractional, Box.h:243-255), so the cells of
// all frames form one array of offsets.
//
// Fused RDF histogram: persistent blocks pull runs of cells from a device work
// counter; a block reloads the frame's box when the frame changes, stages the
// candidate set of the home cell (the (2s + 1)^3 stencil, s = shell, gathered
// as x-row segments so each segment is one contiguous slot range) with each
// candidate's image vector already resolved for queries inside the box, and
// sweeps the cell's queries over it: 32 candidates per warp in registers,
// queries broadcast from shared memory, the exact AABB pair test
// (AABBQuery.cc:93,125) and binning (Histogram.h:327-351) into privatised
// shared histograms, flushed once per block with 64-bit atomics.
//
// Steinhardt neighbours: warp per cell over the 27-cell stencil (staged in
// shared memory, lanes over candidates), count then fill; the bonds of a frame
// batch feed the existing qlm / average / wl kernels over the concatenated
// rows, and the system sums are taken per frame.
#include "fg_batch.cuh"
#include "fg_prof.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

namespace fg {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int BT_TILE = 896;    // staged candidates per tile (four blocks of HistShared fit an SM)
constexpr int BT_QB = 128;      // queries per shared-memory batch
constexpr int BT_ITEMS = 96;    // stencil items: up to 32 rows x 3 x-segments
constexpr int BT_HIST = 2048;   // shared histogram words (all copies)
constexpr int BT_RB_WORDS = 1792; // exact r^2 -> bin table (thresholds + keys)
constexpr int IV_INVALID = 255;    // staged candidate whose image (queries inside the box) is beyond +-1
constexpr int BT_CHUNK_MAX = 4; // cells per work-counter pop (fewer for small grids)

// Largest f with base[f] <= x (base[0] = 0 <= x < base[nframes]).
__device__ __forceinline__ uint32_t frame_of(const uint32_t* __restrict__ base, uint32_t nframes, uint32_t x)
{
    uint32_t lo = 0, hi = nframes;
    while (hi - lo > 1)
    {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(base + mid) <= x)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__global__ void k_frames_assign(const FrameDesc* __restrict__ fd, const uint32_t* __restrict__ pt_base,
                                uint32_t nframes, const float* __restrict__ pts, uint32_t n,
                                uint32_t* __restrict__ cell_of, uint32_t* __restrict__ rank, float4* __restrict__ pos4,
                                uint32_t* __restrict__ cell_count, int* __restrict__ frame_out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t fi = frame_of(pt_base, nframes, i);
        const FrameDesc& F = fd[fi];
        const float x = pts[3 * (size_t) i];
        const float y = pts[3 * (size_t) i + 1];
        const float z = pts[3 * (size_t) i + 2];
        const int dim[3] = {F.dim[0], F.dim[1], F.dim[2]};
        int cx, cy, cz, img;
        point_cell(F.b, dim, x, y, z, cx, cy, cz, img);
        const uint32_t cell = F.cell_base + static_cast<uint32_t>(cx + dim[0] * (cy + dim[1] * cz));
        cell_of[i] = cell;
        rank[i] = atomicAdd(&cell_count[cell], 1u);
        pos4[i] = make_float4(x, y, F.b.is2d ? 0.0f : z, __int_as_float(img));
        if (img != 0 && frame_out[fi] == 0)
            atomicOr(&frame_out[fi], 1);
    }
}

__global__ void k_frames_scatter(uint32_t n, const uint32_t* __restrict__ cell_of, const uint32_t* __restrict__ rank,
                                 const float4* __restrict__ pos4, const uint32_t* __restrict__ start,
                                 float4* __restrict__ cpos, uint32_t* __restrict__ cidx)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const uint32_t pos = start[cell_of[i]] + rank[i];
        cpos[pos] = pos4[i];
        cidx[pos] = i;
    }
}

// ---------------------------------------------------------------------------
// Fused histogram
// ---------------------------------------------------------------------------

struct BItems
{
    uint32_t start[BT_ITEMS];
    uint32_t off[BT_ITEMS + 1];
    int wrap[BT_ITEMS];
    unsigned char home[BT_ITEMS]; // 1: the home cell (half-stencil mode: pairs j > i only)
};

struct HistShared
{
    float4 pos[BT_TILE];        // candidate position, w = packed integer image
    unsigned short lst[8][BT_TILE]; // octant lists: positions of the candidates near each octant
    uint32_t j[BT_TILE];        // global point index
    unsigned char ivc[BT_TILE]; // image for queries inside the box: (kx+1)*9 + (ky+1)*3 + (kz+1), IV_INVALID beyond +-1
    unsigned char wr[BT_TILE];  // cell wrap code (wx + 1) + 3 (wy + 1) + 9 (wz + 1)
    unsigned char home[BT_TILE]; // candidate of the home cell (half-stencil mode)
    float4 q[BT_QB];            // the query block, grouped by octant; w = point index (bits)
    uint32_t qi[BT_QB];
    int qimg[BT_QB];            // packed integer image of each query
    uint32_t qo[9];             // octant o's queries: q[qo[o], qo[o + 1])
    uint32_t lcnt[8];           // octant list lengths
    BItems it;
    DevBox box;
    float4 img4[27];            // box.img as float4 (one shared load per candidate)
    int dim[3];
    int shell;
    uint32_t cell_base;
    uint32_t work;
    uint32_t nkeep;             // candidates kept in the current tile
    float qbox[8][6];           // per-warp bounds of the cell's queries (lo xyz, hi xyz)
    float qfin[6];              // their union
    int qout;                   // some query of the cell lies outside the box
    int sym;                    // half-stencil mode for the current frame
    uint32_t hist[BT_HIST];
    uint32_t rb[BT_RB_WORDS];   // HistParams::rb, when given
};

// Stencil items of local cell c (run by one warp): lane = one (dy, dz) row of
// the (2s + 1)-wide stencil, split into up to three x-segments by wrap. Each
// unwrapped cell offset maps to exactly one (cell, wrap) pair because every
// periodic axis has at least s cells.
__device__ void frame_items(const HistShared& S, const uint32_t* __restrict__ start, int c, BItems& it, int lane)
{
    const int d0 = S.dim[0], d1 = S.dim[1], d2 = S.dim[2];
    const int cz = c / (d0 * d1);
    const int cy = (c / d0) % d1;
    const int cx = c % d0;
    const int s = S.shell;
    const int w = 2 * s + 1;
    const int nrows = S.box.is2d ? w : w * w;
    uint32_t st[3] = {0u, 0u, 0u}, cnt[3] = {0u, 0u, 0u};
    int wc[3] = {13, 13, 13};
    bool home0 = false;
    if (lane < nrows)
    {
        const int dy = lane % w - s;
        const int dz = S.box.is2d ? 0 : lane / w - s;
        const int uy = cy + dy, uz = cz + dz;
        const int wy = uy < 0 ? -1 : (uy >= d1 ? 1 : 0);
        const int wz = uz < 0 ? -1 : (uz >= d2 ? 1 : 0);
        const int row = d0 * ((uy - wy * d1) + d1 * (uz - wz * d2));
        const int x0 = cx - s, x1 = cx + s;
        int lo[3] = {x0 + d0, max(x0, 0), 0};
        int hi[3] = {x0 < 0 ? d0 - 1 : -1, min(x1, d0 - 1), x1 >= d0 ? x1 - d0 : -1};
        int xw[3] = {0, 1, 2}; // x-wrap code of each segment
        if (S.sym)
        {
            // half stencil: rows after the home row whole, the home row from the home
            // cell on (home cell alone, then the cells after it, then those wrapped)
            const bool after = dz > 0 || (dz == 0 && dy > 0);
            const bool before = dz < 0 || (dz == 0 && dy < 0);
            if (before)
            {
                hi[0] = hi[1] = hi[2] = -1;
            }
            else if (!after)
            {
                lo[0] = cx;
                hi[0] = cx;
                xw[0] = 1;
                lo[1] = cx + 1;
                hi[1] = min(x1, d0 - 1);
                xw[1] = 1;
                lo[2] = 0;
                hi[2] = x1 >= d0 ? x1 - d0 : -1;
                xw[2] = 2;
                home0 = true;
            }
        }
#pragma unroll
        for (int k = 0; k < 3; ++k)
        {
            if (lo[k] <= hi[k])
            {
                const uint32_t base = S.cell_base + static_cast<uint32_t>(row);
                st[k] = start[base + lo[k]];
                cnt[k] = start[base + hi[k] + 1] - st[k];
                wc[k] = xw[k] + 3 * (wy + 1) + 9 * (wz + 1);
            }
        }
    }
    const uint32_t tot = cnt[0] + cnt[1] + cnt[2];
    uint32_t incl = tot;
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (lane >= o)
            incl += v;
    }
    uint32_t off = incl - tot;
#pragma unroll
    for (int k = 0; k < 3; ++k)
    {
        it.start[3 * lane + k] = st[k];
        it.off[3 * lane + k] = off;
        it.wrap[3 * lane + k] = wc[k];
        it.home[3 * lane + k] = static_cast<unsigned char>(home0 && k == 0);
        off += cnt[k];
    }
    if (lane == 31)
        it.off[BT_ITEMS] = incl;
}

__device__ __forceinline__ int bitem_of(const BItems& it, uint32_t t)
{
    int s = 0;
#pragma unroll
    for (int step = 64; step >= 1; step >>= 1)
    {
        if (s + step < BT_ITEMS && it.off[s + step] <= t)
            s += step;
    }
    return s;
}

// (shared memory holds four blocks per SM: registers up to that occupancy)
template<int WARPS, int COPIES>
__global__ void __launch_bounds__(WARPS * 32, 4)
    k_frames_hist(BatchGrid g, BallParams p, HistParams h, uint32_t cell_limit, uint32_t chunk,
                  uint32_t* __restrict__ queue, unsigned long long* __restrict__ hist, int sym_ok)
{
    constexpr int THREADS = WARPS * 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    HistShared& S = *reinterpret_cast<HistShared*>(smem_raw);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const bool smem_hist = h.bins * COPIES <= static_cast<uint32_t>(BT_HIST);
    uint32_t* my_hist = S.hist + (warp % COPIES) * h.bins;
    // exclude_ii without a per-pair index test: a query's own point is one of its
    // candidates (home cell, image 0), so r = p - (p + 0) = 0 and the pair test
    // accepts it exactly when r_min = 0; it then lands in bin 0 when the histogram
    // starts at 0. Those self pairs - one per query - are taken back per cell.
    // Bonds to other images of the query's own point are beyond r_max (2 r_max is
    // below every nearest-plane distance), so no other pair carries j == i.
    const bool self_in_bin0 = p.exclude_ii && p.r_min_sq <= 0.0f && h.h_min <= 0.0f && h.h_max > 0.0f;
    const bool test_ii = p.exclude_ii && !self_in_bin0;

    if (smem_hist)
    {
        for (uint32_t t = tid; t < h.bins * COPIES; t += THREADS)
            S.hist[t] = 0;
    }
    // exact r^2 -> bin table: bin = key's first bin + (r^2 >= the next two
    // thresholds); no square root or float-to-int conversion per pair
    const bool rbins = h.rb != nullptr;
    if (rbins)
    {
        for (uint32_t t = tid; t < h.rb_words; t += THREADS)
            S.rb[t] = h.rb[t];
    }
    const float* rb_thr = reinterpret_cast<const float*>(S.rb);
    // counted pairs: ua <= r^2 bits < ua + uspan (r^2 >= +0, so the bit patterns
    // order like the values): the table's folded range, else [r_min^2, r_max^2)
    const uint32_t ua = __float_as_uint(h.rb != nullptr ? h.rb_a : p.r_min_sq);
    const uint32_t ub = __float_as_uint(h.rb != nullptr ? h.rb_b : p.r_max_sq);
    const uint32_t uspan = ub > ua ? ub - ua : 0u;
    const unsigned short* rb_key = reinterpret_cast<const unsigned short*>(S.rb + h.bins + 2);
    int cur_frame = -1;
    float cull2 = 0.0f;
    __syncthreads();

    for (;;)
    {
        if (tid == 0)
            S.work = atomicAdd(queue, chunk);
        __syncthreads();
        const uint32_t c0 = S.work;
        __syncthreads();
        if (c0 >= cell_limit)
            break;
        const uint32_t c1 = min(c0 + chunk, cell_limit);
        for (uint32_t c = c0; c < c1; ++c)
        {
            const uint32_t q0 = g.start[c];
            const uint32_t nqc = g.start[c + 1] - q0;
            if (nqc == 0)
                continue;
            const int f = static_cast<int>(frame_of(g.cell_base, g.nframes, c));
            if (f != cur_frame)
            {
                // block-uniform: every thread walks the same cells; all threads
                // have passed the previous cell's final barrier
                cur_frame = f;
                const FrameDesc& F = g.fd[f];
                const int* src = reinterpret_cast<const int*>(&F.b);
                int* dst = reinterpret_cast<int*>(&S.box);
                for (int t = tid; t < static_cast<int>(sizeof(DevBox) / sizeof(int)); t += THREADS)
                    dst[t] = src[t];
                if (tid < 27)
                    S.img4[tid] = make_float4(F.b.img[tid][0], F.b.img[tid][1], F.b.img[tid][2], 0.0f);
                if (tid == 0)
                {
                    S.dim[0] = F.dim[0];
                    S.dim[1] = F.dim[1];
                    S.dim[2] = F.dim[2];
                    S.shell = F.shell;
                    S.cell_base = F.cell_base;
                    // half stencil: every point of the frame in the box (image 0)
                    S.sym = sym_ok && g.frame_out[f] == 0;
                }
                // candidate cull radius of this frame: r_max plus a margin bounding the
                // difference between the shifted float distance and the exact one
                const float lmax = fmaxf(fmaxf(F.b.L[0], F.b.L[1]), F.b.L[2]) *
                    (1.0f + fabsf(F.b.xy) + fabsf(F.b.xz) + fabsf(F.b.yz));
                const float rmax = sqrtf(p.r_max_sq);
                const float ro = rmax + 2e-5f * (lmax + rmax) + 1e-6f;
                cull2 = ro * ro * (1.0f + 1e-5f);
                __syncthreads();
            }
            if (warp == 0)
                frame_items(S, g.start, static_cast<int>(c - S.cell_base), S.it, lane);
            {
                // bounds of the cell's queries, for the candidate cull
                float lo[3] = {3e30f, 3e30f, 3e30f}, hi[3] = {-3e30f, -3e30f, -3e30f};
                bool out = false;
                for (uint32_t k = tid; k < nqc; k += THREADS)
                {
                    const float4 qv = g.cpos[q0 + k];
                    out |= __float_as_int(qv.w) != 0;
                    lo[0] = fminf(lo[0], qv.x);
                    lo[1] = fminf(lo[1], qv.y);
                    lo[2] = fminf(lo[2], qv.z);
                    hi[0] = fmaxf(hi[0], qv.x);
                    hi[1] = fmaxf(hi[1], qv.y);
                    hi[2] = fmaxf(hi[2], qv.z);
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
                const bool wout = __any_sync(FULL, out);
                if (lane == 0)
                {
#pragma unroll
                    for (int a = 0; a < 3; ++a)
                    {
                        S.qbox[warp][a] = lo[a];
                        S.qbox[warp][3 + a] = hi[a];
                    }
                }
                if (__syncthreads_or(wout && lane == 0) != 0)
                {
                    if (tid == 0)
                        S.qout = 1;
                }
                else if (tid == 0)
                {
                    S.qout = 0;
                }
                if (tid < 6)
                {
                    float v = S.qbox[0][tid];
                    for (int w = 1; w < WARPS; ++w)
                        v = tid < 3 ? fminf(v, S.qbox[w][tid]) : fmaxf(v, S.qbox[w][tid]);
                    S.qfin[tid] = v;
                }
                __syncthreads();
            }
            // the cull needs every query in the box (image 0); otherwise all candidates stay
            const bool sym = S.sym != 0;
            const bool cull = S.qout == 0 && (!test_ii || sym);
            const uint32_t T = S.it.off[BT_ITEMS];
            // octant lists (cull mode, cells of r_max): the queries' bounds split at
            // their middle into eight boxes; a candidate joins the list of each box it
            // lies within the cull radius of, and a query meets only its own box's
            // list (the cell-wide cull bounds a query's candidates by the whole cell,
            // the octant's by an eighth of it; with cells of r_max / 2 the lists cost
            // more than the pairs they drop)
            const bool oct = cull && S.shell == 1;
            const int G = oct ? 8 : 1;
            float mid[3];
#pragma unroll
            for (int a = 0; a < 3; ++a)
                mid[a] = 0.5f * (S.qfin[a] + S.qfin[3 + a]);
            const unsigned lt = (1u << lane) - 1u;
            for (uint32_t t0 = 0; t0 < T; t0 += BT_TILE)
            {
                const uint32_t TT0 = min(static_cast<uint32_t>(BT_TILE), T - t0);
                if (tid == 0)
                    S.nkeep = 0;
                if (tid < 8)
                    S.lcnt[tid] = 0;
                __syncthreads();
                for (uint32_t base = 0; base < TT0; base += THREADS)
                {
                    const uint32_t tl = base + tid;
                    bool keep = false;
                    float4 pp = make_float4(0.f, 0.f, 0.f, 0.f);
                    float3 iv = make_float3(0.f, 0.f, 0.f);
                    int code = IV_INVALID;
                    uint32_t slot = 0;
                    int wr = 13;
                    unsigned om = 0;
                    int s_item = 0;
                    if (tl < TT0)
                    {
                        const uint32_t t = t0 + tl;
                        s_item = bitem_of(S.it, t);
                        slot = S.it.start[s_item] + (t - S.it.off[s_item]);
                        pp = g.cpos[slot];
                        wr = S.it.wrap[s_item];
                        const int pim = __float_as_int(pp.w);
                        const int kx = img_ax(pim, 0) - (wr % 3 - 1);
                        const int ky = img_ax(pim, 1) - ((wr / 3) % 3 - 1);
                        const int kz = img_ax(pim, 2) - (wr / 9 - 1);
                        if (kx >= -1 && kx <= 1 && ky >= -1 && ky <= 1 && kz >= -1 && kz <= 1)
                        {
                            code = (kx + 1) * 9 + (ky + 1) * 3 + (kz + 1);
                            const float* v = S.box.img[code];
                            iv = make_float3(v[0], v[1], v[2]);
                        }
                        keep = true;
                        if (cull)
                        {
                            // farther than r_max (+ margin) from every query of an octant:
                            // no pair with any of them (invalid images are dropped too)
                            const float sc[3] = {pp.x - iv.x, pp.y - iv.y, pp.z - iv.z};
                            float gl[3], gh[3];
#pragma unroll
                            for (int a = 0; a < 3; ++a)
                            {
                                const float l0 = fmaxf(fmaxf(S.qfin[a] - sc[a], sc[a] - mid[a]), 0.f);
                                const float h0 = fmaxf(fmaxf(mid[a] - sc[a], sc[a] - S.qfin[3 + a]), 0.f);
                                gl[a] = l0 * l0;
                                gh[a] = h0 * h0;
                            }
#pragma unroll
                            for (int o = 0; o < 8; ++o)
                            {
                                const float d2 = ((o & 1) ? gh[0] : gl[0]) + ((o & 2) ? gh[1] : gl[1]) +
                                                 ((o & 4) ? gh[2] : gl[2]);
                                om |= (d2 <= cull2 ? 1u : 0u) << o;
                            }
                            keep = code != IV_INVALID && om != 0;
                            if (!keep)
                                om = 0;
                        }
                    }
                    const unsigned km = __ballot_sync(FULL, keep);
                    uint32_t wbase = 0;
                    if (lane == 0 && km != 0)
                        wbase = atomicAdd(&S.nkeep, static_cast<uint32_t>(__popc(km)));
                    wbase = __shfl_sync(FULL, wbase, 0);
                    const uint32_t idx = wbase + __popc(km & lt);
                    if (keep)
                    {
                        S.pos[idx] = pp;
                        S.ivc[idx] = static_cast<unsigned char>(code);
                        S.j[idx] = g.cidx[slot];
                        S.wr[idx] = static_cast<unsigned char>(wr);
                        S.home[idx] = S.it.home[s_item];
                    }
                    if (oct)
                    {
#pragma unroll
                        for (int o = 0; o < 8; ++o)
                        {
                            const bool in = (om >> o) & 1u;
                            const unsigned gm = __ballot_sync(FULL, in);
                            if (gm == 0)
                                continue;
                            uint32_t gb = 0;
                            if (lane == 0)
                                gb = atomicAdd(&S.lcnt[o], static_cast<uint32_t>(__popc(gm)));
                            gb = __shfl_sync(FULL, gb, 0);
                            if (in)
                                S.lst[o][gb + __popc(gm & lt)] = static_cast<unsigned short>(idx);
                        }
                    }
                }
                __syncthreads();
                const uint32_t TT = S.nkeep;
                for (uint32_t qb0 = 0; qb0 < nqc; qb0 += BT_QB)
                {
                    const uint32_t nb = min(static_cast<uint32_t>(BT_QB), nqc - qb0);
                    __syncthreads();
                    // the block's queries (with octants: grouped by octant, a ballot
                    // counting sort by warp 0)
                    bool out_of_box = false;
                    if (!oct)
                    {
                        for (uint32_t k = tid; k < nb; k += THREADS)
                        {
                            const float4 qv = g.cpos[q0 + qb0 + k];
                            const uint32_t qi = g.cidx[q0 + qb0 + k];
                            S.q[k] = make_float4(qv.x, qv.y, qv.z, __uint_as_float(qi));
                            S.qi[k] = qi;
                            S.qimg[k] = __float_as_int(qv.w);
                            out_of_box |= __float_as_int(qv.w) != 0;
                        }
                        if (tid == 0)
                        {
                            S.qo[0] = 0;
                            S.qo[1] = nb;
                        }
                    }
                    else if (warp == 0)
                    {
                        constexpr int QR = BT_QB / 32;
                        float4 qv[QR];
                        uint32_t qiv[QR];
                        int og[QR];
                        bool qlive[QR];
#pragma unroll
                        for (int r = 0; r < QR; ++r)
                        {
                            const uint32_t k = static_cast<uint32_t>(lane + 32 * r);
                            qlive[r] = k < nb;
                            qv[r] = qlive[r] ? g.cpos[q0 + qb0 + k] : make_float4(0.f, 0.f, 0.f, 0.f);
                            qiv[r] = qlive[r] ? g.cidx[q0 + qb0 + k] : 0u;
                            out_of_box |= qlive[r] && __float_as_int(qv[r].w) != 0;
                            og[r] = oct ? (qv[r].x >= mid[0] ? 1 : 0) + (qv[r].y >= mid[1] ? 2 : 0) +
                                              (qv[r].z >= mid[2] ? 4 : 0)
                                        : 0;
                        }
                        uint32_t qoff = 0;
                        for (int o = 0; o < G; ++o)
                        {
                            if (lane == 0)
                                S.qo[o] = qoff;
#pragma unroll
                            for (int r = 0; r < QR; ++r)
                            {
                                const bool in = qlive[r] && og[r] == o;
                                const unsigned m = __ballot_sync(FULL, in);
                                if (in)
                                {
                                    const uint32_t at = qoff + __popc(m & lt);
                                    S.q[at] = make_float4(qv[r].x, qv[r].y, qv[r].z, __uint_as_float(qiv[r]));
                                    S.qi[at] = qiv[r];
                                    S.qimg[at] = __float_as_int(qv[r].w);
                                }
                                qoff += __popc(m);
                            }
                        }
                        if (lane == 0)
                            S.qo[G] = qoff;
                    }
                    // queries inside the box take a branch-free pair loop: invalid
                    // candidates (image beyond +-1) are moved out of range instead
                    // (half-stencil frames hold no point outside the box and count no
                    // pair of a point with itself)
                    const bool general = (__syncthreads_or(out_of_box) != 0 || test_ii) && !sym;
                    if (!general)
                    {
                        // work items: (octant, chunk of 32 of its candidates) over octants
                        // holding queries
                        uint32_t nchk[8];
                        uint32_t items = 0;
#pragma unroll
                        for (int o = 0; o < 8; ++o)
                        {
                            const uint32_t L = o < G ? (oct ? S.lcnt[o] : TT) : 0u;
                            nchk[o] = (o < G && S.qo[o + 1] > S.qo[o]) ? (L + 31) / 32 : 0u;
                            items += nchk[o];
                        }
                        for (uint32_t item = warp; item < items; item += WARPS)
                        {
                            int o = 0;
                            uint32_t ch = item;
                            if (oct)
                            {
#pragma unroll
                                for (int t = 0; t < 8; ++t)
                                {
                                    if (o == t && ch >= nchk[t])
                                    {
                                        ch -= nchk[t];
                                        o = t + 1;
                                    }
                                }
                            }
                            const uint32_t L = oct ? S.lcnt[o] : TT;
                            const uint32_t k = ch * 32 + lane;
                            float4 pp = make_float4(3e30f, 3e30f, 3e30f, 0.f);
                            float3 iv = make_float3(0.f, 0.f, 0.f);
                            uint32_t jj = 0;
                            bool hm = false;
                            if (k < L)
                            {
                                const uint32_t e = oct ? S.lst[o][k] : k;
                                const int code = S.ivc[e];
                                if (code != IV_INVALID)
                                {
                                    pp = S.pos[e];
                                    const float4 v4 = S.img4[code];
                                    iv = make_float3(v4.x, v4.y, v4.z);
                                }
                                jj = S.j[e];
                                hm = S.home[e] != 0;
                            }
                            const bool zero = iv.x == 0.0f && iv.y == 0.0f && iv.z == 0.0f;
                            const uint32_t wrest = zero ? 2u : 1u; // weight of a pair off the home cell
                            const uint32_t qa = S.qo[o], qz = S.qo[o + 1];
                            auto add = [&](uint32_t bin, uint32_t w) {
                                if (smem_hist)
                                    atomicAdd(&my_hist[bin], w);
                                else
                                    atomicAdd(&hist[bin], static_cast<unsigned long long>(w));
                            };
                            if (rbins)
                            {
                                // exact r^2 -> bin (ok: r_min^2 <= r^2 < r_max^2 and inside the histogram)
                                auto bin_of = [&](float rsq, bool& ok) {
                                    // rb_a <= r^2 < rb_b on the bit patterns (r^2 >= +0)
                                    const uint32_t u = __float_as_uint(rsq);
                                    ok = u - ua < uspan;
                                    const uint32_t key = (ok && u >= h.rb_ut) ? ((u - h.rb_ut) >> h.rb_s) + 1u : 0u;
                                    const uint32_t b0 = rb_key[key];
                                    return b0 + (rsq >= rb_thr[b0 + 1] ? 1u : 0u) + (rsq >= rb_thr[b0 + 2] ? 1u : 0u);
                                };
                                // image 0 for the whole chunk: q + 0 is q (up to the sign of a
                                // zero, which r^2 does not see), so the three additions go.
                                // Half stencil (SYM): a pair of image 0 is tested once and
                                // counted twice - p_i - (p_j + 0) is exactly -(p_j - (p_i + 0)),
                                // so both bonds fall in one bin; home-cell pairs only for j > i;
                                // a pair of image k != 0 is tested from both ends: r_ij =
                                // p_j - (p_i + v_k) and r_ji = p_i - (p_j + v_-k), v_-k = -v_k.
                                auto sweep = [&](auto zero_image, auto half) {
                                    constexpr bool Z = decltype(zero_image)::value;
                                    constexpr bool SYM = decltype(half)::value;
#pragma unroll 4
                                    for (uint32_t qq = qa; qq < qz; ++qq)
                                    {
                                        const float4 q = S.q[qq];
                                        const float rx = __fsub_rn(pp.x, Z ? q.x : __fadd_rn(q.x, iv.x));
                                        const float ry = __fsub_rn(pp.y, Z ? q.y : __fadd_rn(q.y, iv.y));
                                        const float rz = __fsub_rn(pp.z, Z ? q.z : __fadd_rn(q.z, iv.z));
                                        bool ok;
                                        const uint32_t bin = bin_of(dot3(rx, ry, rz), ok);
                                        uint32_t w = 1;
                                        if (SYM)
                                            w = hm ? (jj > __float_as_uint(q.w) ? 2u : 0u) : wrest;
                                        if (ok && w != 0)
                                            add(bin, w);
                                        if (SYM && !Z && !zero)
                                        {
                                            const float sx = __fsub_rn(q.x, __fsub_rn(pp.x, iv.x));
                                            const float sy = __fsub_rn(q.y, __fsub_rn(pp.y, iv.y));
                                            const float sz = __fsub_rn(q.z, __fsub_rn(pp.z, iv.z));
                                            bool ok2;
                                            const uint32_t bin2 = bin_of(dot3(sx, sy, sz), ok2);
                                            if (ok2)
                                                add(bin2, 1u);
                                        }
                                    }
                                };
                                const bool all_zero = __all_sync(FULL, zero);
                                if (sym)
                                {
                                    if (all_zero)
                                        sweep(std::true_type {}, std::true_type {});
                                    else
                                        sweep(std::false_type {}, std::true_type {});
                                }
                                else if (all_zero)
                                {
                                    sweep(std::true_type {}, std::false_type {});
                                }
                                else
                                {
                                    sweep(std::false_type {}, std::false_type {});
                                }
                                continue;
                            }
                            // Histogram.h:327-351 binning of the distance of a pair that passed
                            auto count = [&](float rsq, uint32_t w) {
                                if (rsq < p.r_max_sq && rsq >= p.r_min_sq)
                                {
                                    const float d = __fsqrt_rn(rsq);
                                    if (!(d < h.h_min || d >= h.h_max))
                                    {
                                        uint32_t bin =
                                            static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                                        if (bin == h.bins)
                                            bin = h.bins - 1;
                                        add(bin, w);
                                    }
                                }
                            };
                            // half stencil as in the table path above
                            const bool rev = sym && __any_sync(FULL, !zero);
#pragma unroll 4
                            for (uint32_t qq = qa; qq < qz; ++qq)
                            {
                                const float4 q = S.q[qq];
                                const float rx = __fsub_rn(pp.x, __fadd_rn(q.x, iv.x));
                                const float ry = __fsub_rn(pp.y, __fadd_rn(q.y, iv.y));
                                const float rz = __fsub_rn(pp.z, __fadd_rn(q.z, iv.z));
                                const uint32_t w = sym ? (hm ? (jj > __float_as_uint(q.w) ? 2u : 0u) : wrest) : 1u;
                                if (w != 0)
                                    count(dot3(rx, ry, rz), w);
                                if (rev && !zero)
                                {
                                    const float sx = __fsub_rn(q.x, __fsub_rn(pp.x, iv.x));
                                    const float sy = __fsub_rn(q.y, __fsub_rn(pp.y, iv.y));
                                    const float sz = __fsub_rn(q.z, __fsub_rn(pp.z, iv.z));
                                    count(dot3(sx, sy, sz), 1u);
                                }
                            }
                        }
                        continue;
                    }
                    // general: queries outside the box or the per-pair index test (one
                    // group: the cull, and so the octant lists, are off here)
                    const uint32_t nchunks = (TT + 31) / 32;
                    for (uint32_t ch = warp; ch < nchunks; ch += WARPS)
                    {
                        const uint32_t e = ch * 32 + lane;
                        const bool live = e < TT;
                        float4 pp = make_float4(0.f, 0.f, 0.f, 0.f);
                        float3 iv = make_float3(0.f, 0.f, 0.f);
                        bool valid = false;
                        uint32_t jj = 0xffffffffu;
                        int wr = 13;
                        if (live)
                        {
                            pp = S.pos[e];
                            const int code = S.ivc[e];
                            valid = code != IV_INVALID;
                            if (valid)
                            {
                                const float4 v4 = S.img4[code];
                                iv = make_float3(v4.x, v4.y, v4.z);
                            }
                            jj = S.j[e];
                            wr = S.wr[e];
                        }
#pragma unroll 4
                        for (uint32_t qq = 0; qq < nb; ++qq)
                        {
                            const float4 q = S.q[qq];
                            const int qimg = S.qimg[qq];
                            const bool ok = !(test_ii && jj == S.qi[qq]);
                            bool acc = false;
                            float rsq = 0.f;
                            if (qimg == 0)
                            {
                                if (valid && ok)
                                {
                                    const float rx = __fsub_rn(pp.x, __fadd_rn(q.x, iv.x));
                                    const float ry = __fsub_rn(pp.y, __fadd_rn(q.y, iv.y));
                                    const float rz = __fsub_rn(pp.z, __fadd_rn(q.z, iv.z));
                                    rsq = dot3(rx, ry, rz);
                                    acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                                }
                            }
                            else if (live && ok)
                            {
                                // query outside the box: k = n_j - n_q - wrap
                                const int pim = __float_as_int(pp.w);
                                const int kx = img_ax(pim, 0) - img_ax(qimg, 0) - (wr % 3 - 1);
                                const int ky = img_ax(pim, 1) - img_ax(qimg, 1) - ((wr / 3) % 3 - 1);
                                const int kz = img_ax(pim, 2) - img_ax(qimg, 2) - (wr / 9 - 1);
                                if (kx >= -1 && kx <= 1 && ky >= -1 && ky <= 1 && kz >= -1 && kz <= 1)
                                {
                                    const float* v = S.box.img[(kx + 1) * 9 + (ky + 1) * 3 + (kz + 1)];
                                    const float rx = __fsub_rn(pp.x, __fadd_rn(q.x, v[0]));
                                    const float ry = __fsub_rn(pp.y, __fadd_rn(q.y, v[1]));
                                    const float rz = __fsub_rn(pp.z, __fadd_rn(q.z, v[2]));
                                    rsq = dot3(rx, ry, rz);
                                    acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                                }
                            }
                            if (acc)
                            {
                                const float d = __fsqrt_rn(rsq);
                                if (!(d < h.h_min || d >= h.h_max))
                                {
                                    uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                                    if (bin == h.bins)
                                        bin = h.bins - 1;
                                    if (smem_hist)
                                        atomicAdd(&my_hist[bin], 1u);
                                    else
                                        atomicAdd(&hist[bin], 1ull);
                                }
                            }
                        }
                    }
                }
                __syncthreads();
            }
            if (self_in_bin0 && !sym && tid == 0)
            {
                // one self pair per query of the cell, counted into bin 0 above
                if (smem_hist)
                    S.hist[0] -= nqc;
                else
                    atomicAdd(&hist[0], ~static_cast<unsigned long long>(nqc) + 1ull);
            }
        }
    }
    if (smem_hist)
    {
        __syncthreads();
        for (uint32_t bin = tid; bin < h.bins; bin += THREADS)
        {
            uint32_t v = 0;
#pragma unroll
            for (int k = 0; k < COPIES; ++k)
                v += S.hist[k * h.bins + bin];
            if (v != 0)
                atomicAdd(&hist[bin], static_cast<unsigned long long>(v));
        }
    }
}

// ---------------------------------------------------------------------------
// Steinhardt neighbours (warp per cell, 27-cell stencil of r_max cells)
// ---------------------------------------------------------------------------
//
// A warp takes one home cell at a time (cells strided over the resident warps,
// ascending, so a warp meets each frame once). Its queries are the cell's own
// points, handled in groups of at most 32; for each group the stencil's
// candidates - item s in 0..26 (x fastest), slots in cell order: the fixed
// order in which each query's bonds are written and later summed - are staged in
// shared memory FB_TILE at a time, with the image vector that a query inside the
// box needs already resolved. For each query of the group the lanes test 32
// candidates per round (AABBQuery.cc:93,125 arithmetic); bonds keep candidate
// order. The count pass adds ballots; the fill pass appends each accepted bond
// (output row, p_j - q, r^2, j) to a per-warp queue that is drained 32 entries at
// a time, so the exact box.wrap of Steinhardt.cc:155 (three IEEE divisions) runs
// on full warps.

constexpr int FB_WARPS = 4;
constexpr int FB_THREADS = FB_WARPS * 32;
constexpr int FB_TILE = 128;  // staged candidates per warp
constexpr int FB_QUEUE = 64;  // bond queue entries per warp (drained at 32)
constexpr int FB_K0_OK = 1 << 24; // staged image resolved (query in the box)

template<bool FILL> struct FBWarp
{
    float4 pos[FB_TILE];      // x, y, z, point index (bits)
    float4 img[FB_TILE];      // image vector for a query in the box; w = packed n_j - wrap | FB_K0_OK
    float4 q[32];             // the group's queries (w = packed box image)
    uint32_t qi[32];
    unsigned long long qe[FILL ? FB_QUEUE : 1]; // fill: output row of a queued bond
    float4 qv[FILL ? FB_QUEUE : 1];             // fill: p_j - q (x, y, z), r^2
    uint32_t qj[FILL ? FB_QUEUE : 1];           // fill: neighbour index
    uint32_t it_off[28];      // stencil item offsets (prefix of counts)
    uint32_t it_start[27];    // first slot of the item's cell
    int it_wrap[27];          // (wx + 1) + 3 (wy + 1) + 9 (wz + 1)
};

// ONE (one pass, FILL): no counts and offsets beforehand. Each warp takes chunks of
// the bond arrays from a device counter (*alloc) and places each query's bonds at
// its chunk's cursor; before a query the chunk must hold the cell's candidate
// count, an upper bound on the query's bonds (else the rest of the chunk is left
// and a new one taken). seg[i] / counts[i] receive the query's first bond and its
// bond count. Bonds past cap are not written and a query whose bonds end past cap
// gets count 0 (the caller compares *alloc with cap and reruns the two passes when
// the arrays were too small; the kernels after this one never read past cap). A
// query's bonds keep candidate order, so the per-particle sums downstream are the
// same as with the two passes.
constexpr uint32_t FB_CHUNK = 4096; // bond slots a warp takes at a time (one pass)

template<bool FILL, bool ONE = false>
__global__ void __launch_bounds__(FB_THREADS, FILL ? 8 : 10)
    k_frames_ball(BatchGrid g, BallParams p, uint32_t* __restrict__ counts, const uint64_t* __restrict__ offsets,
                  uint32_t* __restrict__ bj, float4* __restrict__ bvd, uint32_t* __restrict__ seg = nullptr,
                  unsigned long long* __restrict__ alloc = nullptr, unsigned long long cap = 0)
{
    __shared__ FBWarp<FILL> sw[FB_WARPS];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    FBWarp<FILL>& W = sw[warp];
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t nwarps = gridDim.x * FB_WARPS;
    uint32_t c = blockIdx.x * FB_WARPS + warp;
    if (c >= g.ncell)
        return;
    uint32_t f = frame_of(g.cell_base, g.nframes, c);
    uint32_t qn = 0; // queued bonds (fill)
    unsigned long long cur = 0, cend = 0; // one pass: the warp's chunk [cur, cend)

    // drain the first n queued bonds: exact box.wrap of p_j - q in frame f
    auto drain = [&](uint32_t n) {
        if (lane < static_cast<int>(n))
        {
            const DevBox& B = g.fd[f].b;
            const unsigned long long e = W.qe[lane];
            const float4 v = W.qv[lane];
            float wx, wy, wz;
            box_wrap(B, v.x, v.y, v.z, wx, wy, wz);
            if (!ONE || e < cap)
            {
                bj[e] = W.qj[lane];
                bvd[e] = make_float4(wx, wy, wz, __fsqrt_rn(v.w));
            }
        }
        __syncwarp();
    };

    for (; c < g.ncell; c += nwarps)
    {
        const uint32_t q0 = g.start[c];
        const uint32_t nqc = g.start[c + 1] - q0;
        if (nqc == 0)
            continue;
        if (c >= g.cell_base[f + 1])
        {
            if (FILL && qn > 0)
            {
                drain(qn);
                qn = 0;
            }
            while (c >= g.cell_base[f + 1])
                ++f;
        }
        const FrameDesc& F = g.fd[f];
        const int d0 = F.dim[0], d1 = F.dim[1], d2 = F.dim[2];
        const int lc = static_cast<int>(c - F.cell_base);
        const int cz = lc / (d0 * d1);
        const int cy = (lc / d0) % d1;
        const int cx = lc % d0;
        const int nst = F.b.is2d ? 9 : 27;
        // stencil items (lane s < nst), same enumeration as the reference order restated above
        {
            uint32_t cnt = 0, st = 0;
            int wr = 13;
            if (lane < nst)
            {
                const int ux = cx + lane % 3 - 1;
                const int uy = cy + (lane / 3) % 3 - 1;
                const int uz = cz + (F.b.is2d ? 0 : lane / 9 - 1);
                const int wx = ux < 0 ? -1 : (ux >= d0 ? 1 : 0);
                const int wy = uy < 0 ? -1 : (uy >= d1 ? 1 : 0);
                const int wz = uz < 0 ? -1 : (uz >= d2 ? 1 : 0);
                const uint32_t cell = F.cell_base +
                                      static_cast<uint32_t>((ux - wx * d0) + d0 * ((uy - wy * d1) + d1 * (uz - wz * d2)));
                st = g.start[cell];
                cnt = g.start[cell + 1] - st;
                wr = (wx + 1) + 3 * (wy + 1) + 9 * (wz + 1);
            }
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const uint32_t v = __shfl_up_sync(FULL, incl, o);
                if (lane >= o)
                    incl += v;
            }
            if (lane < 27)
            {
                W.it_off[lane] = incl - cnt;
                W.it_start[lane] = st;
                W.it_wrap[lane] = wr;
            }
            if (lane == 26)
                W.it_off[27] = incl;
        }
        __syncwarp();
        const uint32_t T = W.it_off[27];
        const uint32_t ntile = (T + FB_TILE - 1) / FB_TILE;

        for (uint32_t g0 = 0; g0 < nqc; g0 += 32)
        {
            const uint32_t ng = min(32u, nqc - g0);
            uint32_t my_cnt = 0;          // bonds so far of query g0 + lane
            uint64_t my_off = 0;
            if (lane < static_cast<int>(ng))
            {
                const uint32_t i = g.cidx[q0 + g0 + lane];
                W.q[lane] = g.cpos[q0 + g0 + lane];
                W.qi[lane] = i;
                if (FILL && !ONE)
                    my_off = offsets[i];
            }
            // one pass over the cell's tiles for the group: counts only (fill_now
            // false) or counts and bonds
            auto run_tiles = [&](bool fill_now, bool alloc_per_query) {
            for (uint32_t tile = 0; tile < ntile; ++tile)
            {
                const uint32_t t0 = tile * FB_TILE;
                const uint32_t TT = min(static_cast<uint32_t>(FB_TILE), T - t0);
                // stage candidates [t0, t0 + TT) unless this tile is already staged
                if (ntile > 1 || g0 == 0)
                {
                    __syncwarp();
                    for (uint32_t tl = lane; tl < TT; tl += 32)
                    {
                        const uint32_t t = t0 + tl;
                        int s = 0;
#pragma unroll
                        for (int step = 16; step >= 1; step >>= 1)
                        {
                            if (s + step < 27 && W.it_off[s + step] <= t)
                                s += step;
                        }
                        const uint32_t slot = W.it_start[s] + (t - W.it_off[s]);
                        const float4 pp = g.cpos[slot];
                        const uint32_t j = g.cidx[slot];
                        const int wr = W.it_wrap[s];
                        const int pim = __float_as_int(pp.w);
                        const int kx = img_ax(pim, 0) - (wr % 3 - 1);
                        const int ky = img_ax(pim, 1) - ((wr / 3) % 3 - 1);
                        const int kz = img_ax(pim, 2) - (wr / 9 - 1);
                        int k0 = pack_image(kx, ky, kz);
                        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (kx >= -1 && kx <= 1 && ky >= -1 && ky <= 1 && kz >= -1 && kz <= 1)
                        {
                            const float* iv = F.b.img[(kx + 1) * 9 + (ky + 1) * 3 + (kz + 1)];
                            v.x = iv[0];
                            v.y = iv[1];
                            v.z = iv[2];
                            k0 |= FB_K0_OK;
                        }
                        v.w = __int_as_float(k0);
                        W.pos[tl] = make_float4(pp.x, pp.y, pp.z, __uint_as_float(j));
                        W.img[tl] = v;
                    }
                    __syncwarp();
                }
                for (uint32_t k = 0; k < ng; ++k)
                {
                    const float4 q = W.q[k];
                    const uint32_t qi = W.qi[k];
                    const int qimg = __float_as_int(q.w);
                    uint32_t base = __shfl_sync(FULL, my_cnt, k);
                    uint64_t off = FILL && !ONE ? __shfl_sync(FULL, my_off, k) : 0;
                    if (ONE && alloc_per_query)
                    {
                        // room for every candidate of the cell (bound on the bonds)
                        if (cend - cur < T)
                        {
                            const unsigned long long want = T > FB_CHUNK ? T : FB_CHUNK;
                            unsigned long long b0 = 0;
                            if (lane == 0)
                                b0 = atomicAdd(alloc, want);
                            cur = __shfl_sync(FULL, b0, 0);
                            cend = cur + want;
                        }
                        if (lane == static_cast<int>(k))
                            my_off = cur;
                    }
                    if (ONE)
                        off = __shfl_sync(FULL, my_off, k);
                    for (uint32_t r0 = 0; r0 < TT; r0 += 32)
                    {
                        const uint32_t tl = r0 + lane;
                        bool acc = false;
                        float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
                        float rsq = 0.f;
                        if (tl < TT)
                        {
                            a = W.pos[tl];
                            const float4 v = W.img[tl];
                            const int k0 = __float_as_int(v.w);
                            float ix = v.x, iy = v.y, iz = v.z;
                            bool ok = (k0 & FB_K0_OK) != 0;
                            if (qimg != 0)
                            {
                                // query outside the box: image k = n_j - n_q - wrap
                                const int kx = img_ax(k0, 0) - img_ax(qimg, 0);
                                const int ky = img_ax(k0, 1) - img_ax(qimg, 1);
                                const int kz = img_ax(k0, 2) - img_ax(qimg, 2);
                                ok = kx >= -1 && kx <= 1 && ky >= -1 && ky <= 1 && kz >= -1 && kz <= 1;
                                if (ok)
                                {
                                    const float* iv = F.b.img[(kx + 1) * 9 + (ky + 1) * 3 + (kz + 1)];
                                    ix = iv[0];
                                    iy = iv[1];
                                    iz = iv[2];
                                }
                            }
                            if (ok && !(p.exclude_ii && __float_as_uint(a.w) == qi))
                            {
                                const float rx = __fsub_rn(a.x, __fadd_rn(q.x, ix));
                                const float ry = __fsub_rn(a.y, __fadd_rn(q.y, iy));
                                const float rz = __fsub_rn(a.z, __fadd_rn(q.z, iz));
                                rsq = dot3(rx, ry, rz);
                                acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                            }
                        }
                        const unsigned bal = __ballot_sync(FULL, acc);
                        if (FILL && fill_now && bal != 0)
                        {
                            if (acc)
                            {
                                const uint32_t slot = qn + __popc(bal & lt);
                                W.qe[slot] = off + base + __popc(bal & lt);
                                W.qv[slot] = make_float4(__fsub_rn(a.x, q.x), __fsub_rn(a.y, q.y),
                                                         __fsub_rn(a.z, q.z), rsq);
                                W.qj[slot] = __float_as_uint(a.w);
                            }
                            qn += __popc(bal);
                            __syncwarp();
                            if (qn >= 32)
                            {
                                drain(32);
                                const uint32_t rest = qn - 32;
                                unsigned long long e = 0;
                                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                                uint32_t j = 0;
                                if (lane < static_cast<int>(rest))
                                {
                                    e = W.qe[32 + lane];
                                    v = W.qv[32 + lane];
                                    j = W.qj[32 + lane];
                                }
                                __syncwarp();
                                if (lane < static_cast<int>(rest))
                                {
                                    W.qe[lane] = e;
                                    W.qv[lane] = v;
                                    W.qj[lane] = j;
                                }
                                __syncwarp();
                                qn = rest;
                            }
                        }
                        base += __popc(bal);
                    }
                    if (lane == static_cast<int>(k))
                        my_cnt = base;
                    if (ONE && alloc_per_query)
                        cur += base; // the query's bonds are placed: advance the cursor
                }
            }
            };
            if (!ONE)
            {
                run_tiles(FILL, false);
            }
            else if (ntile == 1)
            {
                // every candidate in one tile: each query's bonds are found in one
                // sweep, placed at the cursor with room for all candidates
                run_tiles(true, true);
            }
            else
            {
                // several tiles: count the group's bonds, place the group, then fill
                run_tiles(false, false);
                uint32_t incl = lane < static_cast<int>(ng) ? my_cnt : 0u;
                const uint32_t mine = incl;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1)
                {
                    const uint32_t v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= o)
                        incl += v;
                }
                const unsigned long long tot = __shfl_sync(FULL, incl, 31);
                if (cend - cur < tot)
                {
                    const unsigned long long want = tot > FB_CHUNK ? tot : FB_CHUNK;
                    unsigned long long b0 = 0;
                    if (lane == 0)
                        b0 = atomicAdd(alloc, want);
                    cur = __shfl_sync(FULL, b0, 0);
                    cend = cur + want;
                }
                my_off = cur + (incl - mine);
                cur += tot;
                my_cnt = 0;
                run_tiles(true, false);
            }
            if ((!FILL || ONE) && lane < static_cast<int>(ng))
            {
                // one pass: a query whose bonds do not fit below cap gets no bonds,
                // so the kernels after this one read nothing past the arrays (the
                // caller reruns the two passes)
                const bool fits = !ONE || my_off + my_cnt <= cap;
                counts[W.qi[lane]] = fits ? my_cnt : 0u;
                if (ONE)
                    seg[W.qi[lane]] = fits ? static_cast<uint32_t>(my_off) : 0u;
            }
            __syncwarp();
        }
    }
    if (FILL && qn > 0)
        drain(qn);
}

// ---------------------------------------------------------------------------
// Per-frame system sums
// ---------------------------------------------------------------------------

// hi + lo += v with the rounding error of hi + v kept exactly (TwoSum).
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float v)
{
    const float s = __fadd_rn(hi, v);
    const float bp = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(v, bp));
    hi = s;
    lo = __fadd_rn(lo, err);
}

// Rows [r0, r1) of one frame split. For each l, the (row, m) block of qlm is read
// with consecutive threads on consecutive values (thread t: column t mod (2l+1),
// row offset t div (2l+1), rows advancing by 256 div (2l+1)): coalesced loads. Each
// thread keeps float-float running sums (hi + lo, every addition an exact two-sum,
// Knuth's TwoSum: about 48 significant bits, far below the float32 inputs' own
// rounding, on the FP32 pipe instead of GB300's slow FP64 one); the threads of a
// column are then added in FP64 in a fixed order through shared memory and
// partial[f][split][col] is written (the same order every run).
__global__ void __launch_bounds__(256)
    k_frames_sys(const uint32_t* __restrict__ pt_base, StLs ls, int stride, int splits,
                 const float2* __restrict__ src, double* __restrict__ partial)
{
    __shared__ double s_re[256];
    __shared__ double s_im[256];
    const uint32_t f = blockIdx.x;
    const uint32_t split = blockIdx.y;
    const uint32_t r_lo = pt_base[f];
    const uint32_t nf = pt_base[f + 1] - r_lo;
    const uint32_t per = (nf + splits - 1) / splits;
    const uint32_t r0 = r_lo + min(nf, split * per);
    const uint32_t r1 = r_lo + min(nf, (split + 1) * per);
    const int t = threadIdx.x;
    int col0 = 0;
    for (int k = 0; k < ls.nl; ++k)
    {
        const int nm = 2 * ls.l[k] + 1;
        const int rows_per_pass = blockDim.x / nm;
        const int m = t % nm;
        const int rr = t / nm;
        float hr = 0.f, lr = 0.f, hi = 0.f, li = 0.f;
        if (rr < rows_per_pass)
        {
            const float2* base = src + ls.qlm_offset[k];
            for (uint32_t r = r0 + rr; r < r1; r += rows_per_pass)
            {
                const float2 v = base[static_cast<size_t>(r) * nm + m];
                two_sum_acc(hr, lr, v.x);
                two_sum_acc(hi, li, v.y);
            }
        }
        s_re[t] = static_cast<double>(hr) + static_cast<double>(lr);
        s_im[t] = static_cast<double>(hi) + static_cast<double>(li);
        __syncthreads();
        if (t < nm)
        {
            double ar = 0.0, ai = 0.0;
            for (int q = 0; q < rows_per_pass; ++q)
            {
                ar += s_re[q * nm + t];
                ai += s_im[q * nm + t];
            }
            double* out = partial + ((static_cast<size_t>(f) * splits + split) * stride + col0 + t) * 2;
            out[0] = ar;
            out[1] = ai;
        }
        __syncthreads();
        col0 += nm;
    }
}

// Blocks of 8 columns per frame, warp per column: the split sums reduced by lanes
// (every 32nd split) and a fixed shuffle tree (the same order every run), divided
// by n_f.
__global__ void __launch_bounds__(256)
    k_frames_sys_final(const uint32_t* __restrict__ pt_base, int stride, int splits,
                       const double* __restrict__ partial, double* __restrict__ sys)
{
    const uint32_t f = blockIdx.x;
    const int lane = threadIdx.x & 31;
    const int warps = blockDim.x >> 5;
    const double nf = static_cast<double>(pt_base[f + 1] - pt_base[f]);
    for (int col = blockIdx.y * warps + (threadIdx.x >> 5); col < stride; col += warps * gridDim.y)
    {
        double sr = 0.0, si = 0.0;
        for (int k = lane; k < splits; k += 32)
        {
            const double* v = partial + ((static_cast<size_t>(f) * splits + k) * stride + col) * 2;
            sr += v[0];
            si += v[1];
        }
        for (int o = 16; o > 0; o >>= 1)
        {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0)
        {
            sys[2 * (static_cast<size_t>(f) * stride + col)] = nf > 0.0 ? sr / nf : 0.0;
            sys[2 * (static_cast<size_t>(f) * stride + col) + 1] = nf > 0.0 ? si / nf : 0.0;
        }
    }
}

int grid_blocks(size_t n, int threads)
{
    size_t b = (n + threads - 1) / threads;
    if (b > 152 * 32)
        b = 152 * 32;
    return b < 1 ? 1 : static_cast<int>(b);
}

int sms()
{
    static int v = 0;
    if (v == 0)
    {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        if (v <= 0)
            v = 1;
    }
    return v;
}

template<int WARPS, int COPIES>
void hist_launch(const BatchGrid& g, const BallParams& p, const HistParams& h, uint32_t cell_limit, uint32_t* queue,
                 unsigned long long* hist, cudaStream_t s)
{
    const size_t smem = sizeof(HistShared);
    static bool attr = false;
    static int per_sm = 1;
    if (!attr)
    {
        cudaFuncSetAttribute(k_frames_hist<WARPS, COPIES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(smem));
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_frames_hist<WARPS, COPIES>, WARPS * 32, smem);
        if (per_sm < 1)
            per_sm = 1;
        attr = true;
    }
    // runs of up to 4 cells per pop, fewer when the grid is small: at least ~16
    // pops per resident block keep every SM busy to the end
    const uint32_t resident = static_cast<uint32_t>(sms() * per_sm);
    const uint32_t chunk =
        std::max<uint32_t>(1u, std::min<uint32_t>(BT_CHUNK_MAX, cell_limit / std::max<uint32_t>(1u, resident * 16)));
    const uint32_t blocks = std::min<uint32_t>(resident, std::max<uint32_t>(1u, (cell_limit + chunk - 1) / chunk));
    // each unordered pair once where the queries are the points (exclude_ii;
    // frames with a point outside the box keep the whole stencil)
    const int sym_ok = p.exclude_ii ? 1 : 0;
    ProfScope prof_(sym_ok ? (h.rb != nullptr ? "k_frames_hist<half, r2 table>" : "k_frames_hist<half>")
                           : "k_frames_hist", s);
    k_frames_hist<WARPS, COPIES><<<blocks, WARPS * 32, smem, s>>>(g, p, h, cell_limit, chunk, queue, hist, sym_ok);
}

} // namespace

void launch_frames_assign(const FrameDesc* fd, const uint32_t* pt_base, uint32_t nframes, const float* pts, uint32_t n,
                          uint32_t* cell_of, uint32_t* rank, float4* pos4, uint32_t* cell_count, int* frame_out,
                          cudaStream_t s)
{
    if (n == 0)
        return;
    ProfScope prof_("k_frames_assign", s);
    k_frames_assign<<<grid_blocks(n, 256), 256, 0, s>>>(fd, pt_base, nframes, pts, n, cell_of, rank, pos4, cell_count,
                                                         frame_out);
}

void launch_frames_scatter(uint32_t n, const uint32_t* cell_of, const uint32_t* rank, const float4* pos4,
                           const uint32_t* start, float4* cpos, uint32_t* cidx, cudaStream_t s)
{
    if (n == 0)
        return;
    ProfScope prof_("k_frames_scatter", s);
    k_frames_scatter<<<grid_blocks(n, 256), 256, 0, s>>>(n, cell_of, rank, pos4, start, cpos, cidx);
}

size_t frames_hist_smem_bytes()
{
    return sizeof(HistShared);
}

void launch_frames_hist(const BatchHistConfig& cfg, const BatchGrid& g, const BallParams& p, const HistParams& h,
                        uint32_t cell_limit, uint32_t* queue, unsigned long long* hist, cudaStream_t s)
{
    if (cell_limit == 0)
        return;
    // copies == warps: a histogram per warp (no two warps add into one bin), when
    // every copy fits the shared histogram
    const bool per_warp = cfg.copies == cfg.warps && h.bins * static_cast<uint32_t>(cfg.warps) <= BT_HIST;
    if (cfg.warps == 4)
    {
        if (per_warp)
            hist_launch<4, 4>(g, p, h, cell_limit, queue, hist, s);
        else if (cfg.copies == 2)
            hist_launch<4, 2>(g, p, h, cell_limit, queue, hist, s);
        else
            hist_launch<4, 1>(g, p, h, cell_limit, queue, hist, s);
    }
    else
    {
        if (per_warp)
            hist_launch<8, 8>(g, p, h, cell_limit, queue, hist, s);
        else if (cfg.copies == 2)
            hist_launch<8, 2>(g, p, h, cell_limit, queue, hist, s);
        else
            hist_launch<8, 1>(g, p, h, cell_limit, queue, hist, s);
    }
}

namespace {
// one wave of resident blocks, or fewer when the grid has few cells
template<typename K> uint32_t frames_ball_blocks(K kernel, uint32_t ncell)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, FB_THREADS, 0);
    const uint32_t want = static_cast<uint32_t>(sms()) * static_cast<uint32_t>(std::max(per_sm, 1));
    return std::max(1u, std::min<uint32_t>(want, (ncell + FB_WARPS - 1) / FB_WARPS));
}
} // namespace

void launch_frames_ball_count(const BatchGrid& g, const BallParams& p, uint32_t n, uint32_t* counts, cudaStream_t s)
{
    if (n == 0 || g.ncell == 0)
        return;
    const uint32_t blocks = frames_ball_blocks(k_frames_ball<false>, g.ncell);
    ProfScope prof_("k_frames_ball<COUNT>", s);
    k_frames_ball<false><<<blocks, FB_THREADS, 0, s>>>(g, p, counts, nullptr, nullptr, nullptr);
}

void launch_frames_ball_fill(const BatchGrid& g, const BallParams& p, uint32_t n, const uint64_t* offsets,
                             uint32_t* bond_j, float4* bond_vd, cudaStream_t s)
{
    if (n == 0 || g.ncell == 0)
        return;
    const uint32_t blocks = frames_ball_blocks(k_frames_ball<true>, g.ncell);
    ProfScope prof_("k_frames_ball<FILL>", s);
    k_frames_ball<true><<<blocks, FB_THREADS, 0, s>>>(g, p, nullptr, offsets, bond_j, bond_vd);
}

uint64_t frames_ball_onepass_slack(uint32_t ncell)
{
    // every warp may leave the rest of its last chunk unused
    return static_cast<uint64_t>(frames_ball_blocks(k_frames_ball<true, true>, ncell)) * FB_WARPS * FB_CHUNK;
}

void launch_frames_ball_onepass(const BatchGrid& g, const BallParams& p, uint32_t n, uint32_t* counts, uint32_t* seg,
                                uint32_t* bond_j, float4* bond_vd, unsigned long long* alloc, uint64_t cap,
                                cudaStream_t s)
{
    if (n == 0 || g.ncell == 0)
        return;
    const uint32_t blocks = frames_ball_blocks(k_frames_ball<true, true>, g.ncell);
    ProfScope prof_("k_frames_ball<ONE>", s);
    k_frames_ball<true, true><<<blocks, FB_THREADS, 0, s>>>(g, p, counts, nullptr, bond_j, bond_vd, seg, alloc, cap);
}

int frames_sys_splits(uint32_t max_rows)
{
    const uint32_t want = (max_rows + FRAME_SYS_ROWS - 1) / FRAME_SYS_ROWS;
    return static_cast<int>(std::min<uint32_t>(std::max<uint32_t>(want, 1u), 65535u));
}

void launch_frames_sys(const uint32_t* pt_base, uint32_t nframes, uint32_t max_rows, const StLs& ls, int stride,
                       const float2* src, double* partial, double* sys, cudaStream_t s)
{
    if (nframes == 0)
        return;
    const int splits = frames_sys_splits(max_rows);
    {
        ProfScope prof_("k_frames_sys", s);
        k_frames_sys<<<dim3(nframes, splits), 256, 0, s>>>(pt_base, ls, stride, splits, src, partial);
    }
    {
        ProfScope prof_("k_frames_sys_final", s);
        k_frames_sys_final<<<dim3(nframes, (stride + 7) / 8), 256, 0, s>>>(pt_base, stride, splits, partial, sys);
    }
}

// ---------------------------------------------------------------------------
// Exact r^2 -> bin tables
//
// A pair is counted into bin F(r^2): the pair test r_min^2 <= r^2 < r_max^2, then
// d = sqrt(r^2) (correctly rounded) and the regular-axis bin of d
// (Histogram.h:327-351). Every step is monotone in r^2, and so in the bits u of
// the non-negative float r^2: the counted pairs are an interval [uA, uB) of bit
// patterns, on which F is non-decreasing. So F is fixed by its thresholds
// T[b] = min{u : F(u) >= b}, found here by bisection over float bit patterns with
// the same float operations the kernels use. The kernel finds F(u) from a key
// table: key 0 covers [uA, T[b0 + 1]) (b0 = F(uA)); key k > 0 covers a run of
// 2^s bit patterns from there, stores F at the run's start, and each run holds at
// most two thresholds (checked here for every run), so F(u) = key value + [u >=
// T[v + 1]] + [u >= T[v + 2]].
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t INF_BITS = 0x7f800000u;

int host_pair_bin(uint32_t u, const HistParams& h, float r_min_sq, float r_max_sq)
{
    float rsq;
    std::memcpy(&rsq, &u, sizeof(float));
    if (!(rsq < r_max_sq && rsq >= r_min_sq))
        return -1;
    const float d = std::sqrt(rsq);
    if (d < h.h_min || d >= h.h_max)
        return -1;
    uint32_t bin = static_cast<uint32_t>(fmul(fsub(d, h.h_min), h.h_inv));
    if (bin == h.bins)
        bin = h.bins - 1;
    return static_cast<int>(bin);
}

// smallest u in [lo, hi) with pred(u), else hi; pred is false then true
template<typename P> uint32_t first_true(uint32_t lo, uint32_t hi, P pred)
{
    while (lo < hi)
    {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (pred(mid))
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

struct RbEntry
{
    uint32_t id[6];
    HistParams h;
};

std::mutex g_rb_mutex;
std::vector<RbEntry> g_rb_cache;
constexpr size_t RB_CACHE_MAX = 256;

float bits_float(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, sizeof(float));
    return f;
}

uint32_t float_bits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, sizeof(float));
    return u;
}

// false when the table does not fit BT_RB_WORDS
bool build_rsq_bins(const HistParams& h, float r_min_sq, float r_max_sq, std::vector<uint32_t>& words,
                    HistParams& out)
{
    const uint32_t bins = h.bins;
    if (bins == 0 || bins + 3 > static_cast<uint32_t>(BT_RB_WORDS))
        return false;
    auto F = [&](uint32_t u) { return host_pair_bin(u, h, r_min_sq, r_max_sq); };
    const uint32_t ua = first_true(0u, INF_BITS + 1, [&](uint32_t u) {
        const float r = bits_float(u);
        return r >= r_min_sq && std::sqrt(r) >= h.h_min;
    });
    const uint32_t ub = first_true(0u, INF_BITS + 1, [&](uint32_t u) {
        const float r = bits_float(u);
        return r >= r_max_sq || std::sqrt(r) >= h.h_max;
    });
    std::vector<uint32_t> thr(bins + 2, INF_BITS);
    std::vector<uint16_t> keys(1, 0);
    uint32_t ut = ub, shift = 31;
    if (ua >= ub)
    {
        // nothing is counted: r^2 >= 0 and r^2 < 0 never both hold
        out.rb_a = 0.0f;
        out.rb_b = 0.0f;
    }
    else
    {
        if (bins > 65535)
            return false;
        thr[0] = ua;
        for (uint32_t b = 1; b < bins; ++b)
            thr[b] = first_true(ua, ub, [&](uint32_t u) { return F(u) >= static_cast<int>(b); });
        const int b0 = F(ua);
        keys[0] = static_cast<uint16_t>(b0);
        ut = static_cast<uint32_t>(b0) + 1 < bins ? thr[b0 + 1] : ub;
        if (ut < ub)
        {
            bool done = false;
            for (int s = 31; s >= 0 && !done; --s)
            {
                const uint64_t nkeys = (static_cast<uint64_t>(ub - 1 - ut) >> s) + 2;
                if (bins + 2 + (nkeys + 1) / 2 > static_cast<uint64_t>(BT_RB_WORDS))
                    return false;
                keys.assign(nkeys, 0);
                keys[0] = static_cast<uint16_t>(b0);
                bool ok = true;
                for (uint64_t k = 1; k < nkeys && ok; ++k)
                {
                    const uint64_t start = ut + ((k - 1) << s);
                    const uint64_t end = std::min<uint64_t>(ut + (k << s), ub) - 1;
                    const int fs = F(static_cast<uint32_t>(start));
                    const int fe = F(static_cast<uint32_t>(end));
                    ok = fs >= 0 && fe >= fs && fe <= fs + 2;
                    keys[k] = static_cast<uint16_t>(fs);
                }
                if (ok)
                {
                    shift = static_cast<uint32_t>(s);
                    done = true;
                }
            }
            if (!done)
                return false;
        }
        out.rb_a = bits_float(ua);
        out.rb_b = bits_float(ub);
    }
    words.assign(bins + 2 + (keys.size() + 1) / 2, 0u);
    std::memcpy(words.data(), thr.data(), sizeof(uint32_t) * thr.size());
    std::memcpy(words.data() + bins + 2, keys.data(), sizeof(uint16_t) * keys.size());
    out.rb_ut = ut;
    out.rb_s = shift;
    out.rb_words = static_cast<uint32_t>(words.size());
    return true;
}

} // namespace

HistParams with_rsq_bins(const HistParams& h, float r_min_sq, float r_max_sq)
{
    const uint32_t id[6] = {float_bits(h.h_min), float_bits(h.h_max), float_bits(h.h_inv), h.bins,
                            float_bits(r_min_sq), float_bits(r_max_sq)};
    std::lock_guard<std::mutex> lock(g_rb_mutex);
    for (const RbEntry& e : g_rb_cache)
    {
        if (std::memcmp(e.id, id, sizeof(id)) == 0)
            return e.h;
    }
    HistParams out = h;
    out.rb = nullptr;
    if (g_rb_cache.size() >= RB_CACHE_MAX)
        return out;
    std::vector<uint32_t> words;
    HistParams t = h;
    if (build_rsq_bins(h, r_min_sq, r_max_sq, words, t))
    {
        void* d = nullptr;
        if (cudaMalloc(&d, sizeof(uint32_t) * words.size()) == cudaSuccess &&
            cudaMemcpy(d, words.data(), sizeof(uint32_t) * words.size(), cudaMemcpyHostToDevice) == cudaSuccess)
        {
            t.rb = static_cast<const uint32_t*>(d);
            out = t;
        }
        else
        {
            if (d != nullptr)
                cudaFree(d);
            cudaGetLastError();
            return out; // not cached: tried again next call
        }
    }
    RbEntry e;
    std::memcpy(e.id, id, sizeof(id));
    e.h = out;
    g_rb_cache.push_back(e);
    return out;
}

} // namespace fg
