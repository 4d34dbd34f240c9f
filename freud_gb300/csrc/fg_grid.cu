// Cell-list build (counting sort of points into cells) and exclusive scans.
//
// Replaces the serial head/next linked list of freud/locality/LinkCell.cc:316-336
// and the serial AABB tree build of freud/locality/AABBQuery.cc:53-69 with a
// data-parallel counting sort: cell index from the exact makeFractional
// arithmetic, per-cell counts by atomics, exclusive scan, scatter into a
// cell-sorted float4 array (x, y, z, packed integer box image) so candidate
// loads in the query kernels are 16-byte and coalesced.
#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

__global__ void k_assign(DevBox b, const float* __restrict__ pts, uint32_t n, int dx, int dy, int dz,
                         uint32_t* __restrict__ cell_of, uint32_t* __restrict__ rank,
                         uint32_t* __restrict__ cell_count)
{
    const int dim[3] = {dx, dy, dz};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        int cx, cy, cz, img;
        point_cell(b, dim, pts[3 * (size_t) i], pts[3 * (size_t) i + 1], pts[3 * (size_t) i + 2], cx, cy, cz,
                   img);
        const uint32_t cell = static_cast<uint32_t>(cx + dx * (cy + dy * cz));
        cell_of[i] = cell;
        rank[i] = atomicAdd(&cell_count[cell], 1u);
    }
}

__global__ void k_scatter(DevBox b, const float* __restrict__ pts, uint32_t n, int dx, int dy, int dz,
                          const uint32_t* __restrict__ cell_of, const uint32_t* __restrict__ rank,
                          const uint32_t* __restrict__ start, float4* __restrict__ cpos,
                          uint32_t* __restrict__ cidx)
{
    const int dim[3] = {dx, dy, dz};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float x = pts[3 * (size_t) i];
        const float y = pts[3 * (size_t) i + 1];
        const float z = pts[3 * (size_t) i + 2];
        int cx, cy, cz, img;
        point_cell(b, dim, x, y, z, cx, cy, cz, img);
        const uint32_t pos = start[cell_of[i]] + rank[i];
        cpos[pos] = make_float4(x, y, b.is2d ? 0.0f : z, __int_as_float(img));
        cidx[pos] = i;
    }
}

static int grid_for(size_t n, int threads)
{
    size_t blocks = (n + threads - 1) / threads;
    if (blocks > 152 * 32)
    {
        blocks = 152 * 32;
    }
    return blocks < 1 ? 1 : static_cast<int>(blocks);
}

void launch_assign(const DevBox& box, const float* pts, uint32_t n, const int dim[3], uint32_t* cell_of,
                   uint32_t* rank, uint32_t* cell_count, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_assign", s);
        k_assign<<<grid_for(n, 256), 256, 0, s>>>(box, pts, n, dim[0], dim[1], dim[2], cell_of, rank, cell_count);
    }
}

void launch_scatter(const DevBox& box, const float* pts, uint32_t n, const uint32_t* cell_of,
                    const uint32_t* rank, const uint32_t* start, float4* cpos, uint32_t* cidx, cudaStream_t s)
{
    // dims are only used to recompute the packed image; any dims give the same image
    if (n == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_scatter", s);
        k_scatter<<<grid_for(n, 256), 256, 0, s>>>(box, pts, n, 1, 1, 1, cell_of, rank, start, cpos, cidx);
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan: per-tile sums -> recursive scan of tile sums -> tile scan.
// ---------------------------------------------------------------------------
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template<typename TI, typename TO> __global__ void k_tile_sums(const TI* __restrict__ in, size_t n, TO* sums)
{
    __shared__ TO warp_sums[SCAN_THREADS / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * SCAN_TILE;
    TO acc = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        const size_t idx = base + static_cast<size_t>(k) * SCAN_THREADS + threadIdx.x;
        if (idx < n)
        {
            acc += static_cast<TO>(in[idx]);
        }
    }
    for (int o = 16; o > 0; o >>= 1)
    {
        acc += __shfl_down_sync(0xffffffffu, acc, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        warp_sums[threadIdx.x >> 5] = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        TO t = 0;
        for (int w = 0; w < SCAN_THREADS / 32; ++w)
        {
            t += warp_sums[w];
        }
        sums[blockIdx.x] = t;
    }
}

// Exclusive scan of one tile with an added base offset (offsets[blockIdx.x] or 0).
template<typename TI, typename TO>
__global__ void k_tile_scan(const TI* __restrict__ in, TO* __restrict__ out, size_t n, const TO* offsets)
{
    __shared__ TO warp_tot[SCAN_THREADS / 32];
    const size_t base = static_cast<size_t>(blockIdx.x) * SCAN_TILE + static_cast<size_t>(threadIdx.x) * SCAN_ITEMS;
    TO v[SCAN_ITEMS];
    TO local = 0;
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        const size_t idx = base + k;
        v[k] = idx < n ? static_cast<TO>(in[idx]) : 0;
        local += v[k];
    }
    // inclusive warp scan of per-thread totals
    TO incl = local;
    const int lane = threadIdx.x & 31;
    for (int o = 1; o < 32; o <<= 1)
    {
        TO t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o)
        {
            incl += t;
        }
    }
    if (lane == 31)
    {
        warp_tot[threadIdx.x >> 5] = incl;
    }
    __syncthreads();
    TO warp_off = 0;
    for (int w = 0; w < static_cast<int>(threadIdx.x >> 5); ++w)
    {
        warp_off += warp_tot[w];
    }
    TO run = (offsets != nullptr ? offsets[blockIdx.x] : 0) + warp_off + incl - local;
    for (int k = 0; k < SCAN_ITEMS; ++k)
    {
        const size_t idx = base + k;
        if (idx < n)
        {
            out[idx] = run;
        }
        run += v[k];
    }
}

size_t scan_scratch_bytes(size_t n)
{
    size_t total = 0;
    size_t m = n;
    while (m > 1)
    {
        m = (m + SCAN_TILE - 1) / SCAN_TILE;
        total += (m + 1) * sizeof(uint64_t) * 2;
    }
    return total + 256;
}

template<typename TI, typename TO> static void scan_impl(const TI* in, TO* out, size_t n, char* scratch, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    const size_t tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (tiles == 1)
    {
        {
            ProfScope prof_("k_tile_scan<TI, TO>", s);
            k_tile_scan<TI, TO><<<1, SCAN_THREADS, 0, s>>>(in, out, n, nullptr);
        }
        return;
    }
    TO* sums = reinterpret_cast<TO*>(scratch);
    TO* sums_scan = sums + tiles + 1;
    char* next = reinterpret_cast<char*>(sums_scan + tiles + 1);
    {
        ProfScope prof_("k_tile_sums<TI, TO>", s);
        k_tile_sums<TI, TO><<<static_cast<unsigned>(tiles), SCAN_THREADS, 0, s>>>(in, n, sums);
    }
    scan_impl<TO, TO>(sums, sums_scan, tiles, next, s);
    {
        ProfScope prof_("k_tile_scan<TI, TO>", s);
        k_tile_scan<TI, TO><<<static_cast<unsigned>(tiles), SCAN_THREADS, 0, s>>>(in, out, n, sums_scan);
    }
}

void scan_u32_to_u32(const uint32_t* in, uint32_t* out, size_t n, void* scratch, cudaStream_t s)
{
    scan_impl<uint32_t, uint32_t>(in, out, n, static_cast<char*>(scratch), s);
}

void scan_u32_to_u64(const uint32_t* in, uint64_t* out, size_t n, void* scratch, cudaStream_t s)
{
    scan_impl<uint32_t, uint64_t>(in, out, n, static_cast<char*>(scratch), s);
}

// ---------------------------------------------------------------------------
// NeighborList helpers
// ---------------------------------------------------------------------------
__global__ void k_fill_f32(float* a, float v, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    {
        a[i] = v;
    }
}

void launch_fill_f32(float* a, float v, uint64_t n, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_fill_f32", s);
        k_fill_f32<<<grid_for(n, 256), 256, 0, s>>>(a, v, n);
    }
}

// flag |= 1 when the n 32-bit words of a and b differ anywhere (bitwise: equal
// words give identical pair arithmetic, so a query whose points equal the
// object's points can run on the object's own grid).
__global__ void k_words_differ(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, uint64_t n,
                               uint32_t* flag)
{
    bool d = false;
    for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
    {
        d |= a[i] != b[i];
    }
    if (__syncthreads_or(d) && threadIdx.x == 0)
    {
        atomicOr(flag, 1u);
    }
}

void launch_words_differ(const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* flag, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_words_differ", s);
        k_words_differ<<<grid_for(n, 256), 256, 0, s>>>(a, b, n, flag);
    }
}

// segments[i] = first bond of query i, counts[i] = its bond count
// (NeighborList::updateSegmentCounts, NeighborList.cc:199-232; queries with no
// bonds keep segment 0 and count 0 as the reference leaves them).
__global__ void k_segments(const uint2* __restrict__ ij, uint64_t nb, uint32_t* segments, uint32_t* counts)
{
    for (uint64_t b = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; b < nb; b += (uint64_t) gridDim.x * blockDim.x)
    {
        const uint32_t i = ij[b].x;
        if (b == 0 || ij[b - 1].x != i)
        {
            segments[i] = static_cast<uint32_t>(b);
            uint64_t e = b + 1;
            while (e < nb && ij[e].x == i)
            {
                ++e;
            }
            counts[i] = static_cast<uint32_t>(e - b);
        }
    }
}

void launch_segments(const uint2* ij, uint64_t nb, uint32_t nq, uint32_t* segments, uint32_t* counts,
                     cudaStream_t s)
{
    cudaMemsetAsync(segments, 0, sizeof(uint32_t) * nq, s);
    cudaMemsetAsync(counts, 0, sizeof(uint32_t) * nq, s);
    if (nb == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_segments", s);
        k_segments<<<grid_for(nb, 256), 256, 0, s>>>(ij, nb, segments, counts);
    }
}

__global__ void k_seg_from_offsets(const uint32_t* __restrict__ counts, const uint64_t* __restrict__ offsets,
                                   uint32_t nq, uint32_t* __restrict__ segments)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x)
    {
        segments[i] = counts[i] != 0 ? static_cast<uint32_t>(offsets[i]) : 0u;
    }
}

void launch_segments_from_offsets(const uint32_t* counts, const uint64_t* offsets, uint32_t nq, uint32_t* segments,
                                  cudaStream_t s)
{
    if (nq == 0)
    {
        return;
    }
    {
        ProfScope prof_("k_seg_from_offsets", s);
        k_seg_from_offsets<<<grid_for(nq, 256), 256, 0, s>>>(counts, offsets, nq, segments);
    }
}

// ---------------------------------------------------------------------------
// Sort the points of every cell by point index (cells of up to SORT_CELL_MAX
// points; larger cells are left in scatter order and never reach the per-cell
// merge, whose candidate capacity they exceed). A home cell's candidate set is
// then a union of runs already sorted by index.
// ---------------------------------------------------------------------------
constexpr int SORT_WARPS = 4;

// Reads the scatter-ordered (cpos_in, cidx_in) and writes every cell's points
// sorted by (point index, scatter slot) to (cpos_out, cidx_out). Cells larger than
// SORT_CELL_MAX are copied in scatter order. A warp takes 4 consecutive cells at
// a time: each 8-lane group ranks the points of a cell of at most 8 (the common
// case for grids of r_max cells at liquid densities) by counting the smaller keys
// of its group; larger cells are then sorted by the whole warp, one at a time.
__global__ void __launch_bounds__(SORT_WARPS * 32)
    k_sort_cells(const uint32_t* __restrict__ start, int ncell, const float4* __restrict__ cpos_in,
                 const uint32_t* __restrict__ cidx_in, float4* __restrict__ cpos_out, uint32_t* __restrict__ cidx_out)
{
    __shared__ unsigned long long s_key[SORT_WARPS][SORT_CELL_MAX];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    unsigned long long* key = s_key[warp];
    // one cell of more than 8 points, by the whole warp
    auto sort_one = [&](uint32_t b0, uint32_t n) {
        if (n > static_cast<uint32_t>(SORT_CELL_MAX))
        {
            for (uint32_t e = lane; e < n; e += 32)
            {
                cpos_out[b0 + e] = cpos_in[b0 + e];
                cidx_out[b0 + e] = cidx_in[b0 + e];
            }
            return;
        }
        if (n <= 32)
        {
            // register bitonic sort over the warp on (index << 32 | slot) keys
            unsigned long long k = lane < static_cast<int>(n)
                ? ((static_cast<unsigned long long>(cidx_in[b0 + lane]) << 32) | static_cast<unsigned>(lane))
                : ~0ull;
            for (int kk = 2; kk <= 32; kk <<= 1)
            {
                for (int j = kk >> 1; j > 0; j >>= 1)
                {
                    const unsigned long long o = __shfl_xor_sync(0xffffffffu, k, j);
                    const bool up = (lane & kk) == 0;
                    const bool lower = (lane & j) == 0;
                    const bool take = lower ? (up ? o < k : o > k) : (up ? o > k : o < k);
                    if (take)
                        k = o;
                }
            }
            if (lane < static_cast<int>(n))
            {
                cpos_out[b0 + lane] = cpos_in[b0 + static_cast<uint32_t>(k & 0xffffffffull)];
                cidx_out[b0 + lane] = static_cast<uint32_t>(k >> 32);
            }
            return;
        }
        uint32_t np2 = 64;
        while (np2 < n)
            np2 <<= 1;
        for (uint32_t e = lane; e < np2; e += 32)
            key[e] = e < n ? ((static_cast<unsigned long long>(cidx_in[b0 + e]) << 32) | e) : ~0ull;
        __syncwarp();
        for (uint32_t kk = 2; kk <= np2; kk <<= 1)
        {
            for (uint32_t j = kk >> 1; j > 0; j >>= 1)
            {
                for (uint32_t e = lane; e < np2 / 2; e += 32)
                {
                    const uint32_t lo = ((e & ~(j - 1)) << 1) | (e & (j - 1));
                    const uint32_t hi = lo | j;
                    const bool up = (lo & kk) == 0;
                    const unsigned long long a = key[lo], c2 = key[hi];
                    if ((a > c2) == up)
                    {
                        key[lo] = c2;
                        key[hi] = a;
                    }
                }
                __syncwarp();
            }
        }
        for (uint32_t e = lane; e < n; e += 32)
        {
            cpos_out[b0 + e] = cpos_in[b0 + static_cast<uint32_t>(key[e] & 0xffffffffull)];
            cidx_out[b0 + e] = static_cast<uint32_t>(key[e] >> 32);
        }
        __syncwarp();
    };
    const int grp = lane >> 3;
    const int e = lane & 7;
    for (int c4 = (blockIdx.x * SORT_WARPS + warp) * 4; c4 < ncell; c4 += gridDim.x * SORT_WARPS * 4)
    {
        const int c = c4 + grp;
        uint32_t b0 = 0, n = 0;
        if (c < ncell)
        {
            b0 = start[c];
            n = start[c + 1] - b0;
        }
        const bool small = n <= 8;
        const uint32_t my = (small && e < static_cast<int>(n)) ? cidx_in[b0 + e] : 0xffffffffu;
        uint32_t rank = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k)
        {
            const uint32_t o = __shfl_sync(0xffffffffu, my, k, 8);
            rank += (o < my || (o == my && k < e)) ? 1u : 0u;
        }
        if (small && e < static_cast<int>(n))
        {
            cpos_out[b0 + rank] = cpos_in[b0 + e];
            cidx_out[b0 + rank] = my;
        }
        unsigned big = __ballot_sync(0xffffffffu, e == 0 && !small);
        while (big != 0)
        {
            const int src = __ffs(big) - 1;
            big &= big - 1u;
            sort_one(__shfl_sync(0xffffffffu, b0, src), __shfl_sync(0xffffffffu, n, src));
        }
    }
}

void launch_sort_cells(const uint32_t* start, int ncell, const float4* cpos_in, const uint32_t* cidx_in,
                       float4* cpos_out, uint32_t* cidx_out, cudaStream_t s)
{
    if (ncell == 0)
    {
        return;
    }
    const int blocks = grid_for(static_cast<size_t>(ncell) * 8, SORT_WARPS * 32);
    {
        ProfScope prof_("k_sort_cells", s);
        k_sort_cells<<<blocks, SORT_WARPS * 32, 0, s>>>(start, ncell, cpos_in, cidx_in, cpos_out, cidx_out);
    }
}

} // namespace fg
