// CellQuery ghost grid (CellQuery.cc:55-176, CellQuery.h:143-167, 218-299).
//
// Every point is placed in a padded axis-aligned grid of cells of width r_cut
// together with its ghost copies: a point within r_cut (in fractional units per
// axis) of a box face gets copies shifted by the lattice vectors across that
// face, edge and corner (up to 7), built in the reference's float operations so
// the ghost positions - and with them the pair vectors g - q - are identical.
// Copies that fall outside the grid are dropped, as the reference drops them.
// A counting sort (atomics per cell, scan, scatter) gives the cell offsets; each
// copy keeps the index of its real point.
#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

constexpr uint32_t NO_CELL = 0xffffffffu;

// Cell of p, or false outside the grid (CellQuery.h:53-75).
__device__ __forceinline__ bool ghost_cell(const GhostParams& P, float x, float y, float z, uint32_t& idx)
{
    const float fx = floorf(__fmul_rn(__fsub_rn(x, P.gmin[0]), P.ginv));
    const float fy = floorf(__fmul_rn(__fsub_rn(y, P.gmin[1]), P.ginv));
    const float fz = floorf(__fmul_rn(__fsub_rn(z, P.gmin[2]), P.ginv));
    if (!(fx >= 0.0f && fy >= 0.0f && fz >= 0.0f && fx < static_cast<float>(P.dim[0])
          && fy < static_cast<float>(P.dim[1]) && fz < static_cast<float>(P.dim[2])))
        return false;
    const int cx = static_cast<int>(fx), cy = static_cast<int>(fy), cz = static_cast<int>(fz);
    idx = static_cast<uint32_t>((cz * P.dim[1] + cy) * P.dim[0] + cx);
    return true;
}

// The copies of one point in the reference's order: ghosts (faces x, y, z,
// edges xy, xz, yz, corner; CellQuery.h:244-296) then the point itself.
__device__ __forceinline__ int point_copies(const GhostParams& P, float x, float y, float z, int with_ghosts,
                                            float3* out)
{
    int n = 0;
    if (with_ghosts)
    {
        float fx, fy, fz;
        make_fractional(P.b, x, y, z, fx, fy, fz);
        // f <= fr in float; f >= 1.0 - fr with the double literal 1.0 (so in double)
        const int dx = static_cast<int>(fx <= P.fr[0]) - static_cast<int>(static_cast<double>(fx) >= 1.0 - static_cast<double>(P.fr[0]));
        const int dy = static_cast<int>(fy <= P.fr[1]) - static_cast<int>(static_cast<double>(fy) >= 1.0 - static_cast<double>(P.fr[1]));
        int dz = static_cast<int>(fz <= P.fr[2]) - static_cast<int>(static_cast<double>(fz) >= 1.0 - static_cast<double>(P.fr[2]));
        if (P.b.is2d)
            dz = 0;
        if (dx != 0 || dy != 0 || dz != 0)
        {
            auto site = [&](int i, int j, int k) {
                float sx = 0.0f, sy = 0.0f, sz = 0.0f;
                const int c[3] = {i, j, k};
#pragma unroll
                for (int a = 0; a < 3; ++a)
                {
                    if (c[a] != 0)
                    {
                        const float s = c[a] == 1 ? 1.0f : -1.0f;
                        sx = __fadd_rn(sx, s * P.lat[a][0]);
                        sy = __fadd_rn(sy, s * P.lat[a][1]);
                        sz = __fadd_rn(sz, s * P.lat[a][2]);
                    }
                }
                out[n++] = make_float3(__fadd_rn(x, sx), __fadd_rn(y, sy), __fadd_rn(z, sz));
            };
            if (dx != 0)
                site(dx, 0, 0);
            if (dy != 0)
                site(0, dy, 0);
            if (dz != 0)
                site(0, 0, dz);
            if (dx != 0 && dy != 0)
                site(dx, dy, 0);
            if (dx != 0 && dz != 0)
                site(dx, 0, dz);
            if (dy != 0 && dz != 0)
                site(0, dy, dz);
            if (dx != 0 && dy != 0 && dz != 0)
                site(dx, dy, dz);
        }
    }
    out[n++] = make_float3(x, y, z);
    return n;
}

__global__ void k_ghost_count(GhostParams P, const float* __restrict__ pts, uint32_t n, int with_ghosts,
                              uint32_t* __restrict__ copy_cell, uint32_t* __restrict__ copy_rank,
                              uint32_t* __restrict__ cell_count)
{
    const uint32_t bucket = static_cast<uint32_t>(P.dim[0] * P.dim[1] * P.dim[2]);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        float3 c[8];
        const int nc = point_copies(P, pts[3 * (size_t) i], pts[3 * (size_t) i + 1], pts[3 * (size_t) i + 2],
                                    with_ghosts, c);
        for (int k = 0; k < 8; ++k)
        {
            uint32_t idx = NO_CELL;
            if (k < nc && !ghost_cell(P, c[k].x, c[k].y, c[k].z, idx))
                idx = with_ghosts ? NO_CELL : bucket;
            if (k >= nc)
                idx = NO_CELL;
            copy_cell[8 * (size_t) i + k] = idx;
            if (idx != NO_CELL)
                copy_rank[8 * (size_t) i + k] = atomicAdd(&cell_count[idx], 1u);
        }
    }
}

__global__ void k_ghost_scatter(GhostParams P, const float* __restrict__ pts, uint32_t n, int with_ghosts,
                                const uint32_t* __restrict__ copy_cell, const uint32_t* __restrict__ copy_rank,
                                const uint32_t* __restrict__ start, float4* __restrict__ cpos,
                                uint32_t* __restrict__ cidx)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        float3 c[8];
        const int nc = point_copies(P, pts[3 * (size_t) i], pts[3 * (size_t) i + 1], pts[3 * (size_t) i + 2],
                                    with_ghosts, c);
        for (int k = 0; k < nc; ++k)
        {
            const uint32_t idx = copy_cell[8 * (size_t) i + k];
            if (idx == NO_CELL)
                continue;
            const uint32_t pos = start[idx] + copy_rank[8 * (size_t) i + k];
            cpos[pos] = make_float4(c[k].x, c[k].y, c[k].z, 0.0f);
            cidx[pos] = i;
        }
    }
}

int ghost_blocks(size_t n)
{
    size_t b = (n + 255) / 256;
    if (b > 152 * 32)
        b = 152 * 32;
    return b < 1 ? 1 : static_cast<int>(b);
}

} // namespace

void launch_ghost_count(const GhostParams& gp, const float* pts, uint32_t n, int with_ghosts, uint32_t* copy_cell,
                        uint32_t* copy_rank, uint32_t* cell_count, cudaStream_t s)
{
    if (n == 0)
        return;
    ProfScope prof_("k_ghost_count", s);
    k_ghost_count<<<ghost_blocks(n), 256, 0, s>>>(gp, pts, n, with_ghosts, copy_cell, copy_rank, cell_count);
}

void launch_ghost_scatter(const GhostParams& gp, const float* pts, uint32_t n, int with_ghosts,
                          const uint32_t* copy_cell, const uint32_t* copy_rank, const uint32_t* start, float4* cpos,
                          uint32_t* cidx, cudaStream_t s)
{
    if (n == 0)
        return;
    ProfScope prof_("k_ghost_scatter", s);
    k_ghost_scatter<<<ghost_blocks(n), 256, 0, s>>>(gp, pts, n, with_ghosts, copy_cell, copy_rank, start, cpos, cidx);
}

} // namespace fg
