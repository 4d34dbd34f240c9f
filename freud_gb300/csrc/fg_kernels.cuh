// Host-side launch interface of the freud_gb300 kernels (implemented in the .cu files).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "fg_common.cuh"

namespace fg {

enum Arith : int
{
    ARITH_AABB = 0, // r = p_j - (q + image)   AABBQuery.cc:93,125 (also RawPoints, the default)
    ARITH_WRAP = 1, // r = box.wrap(p_j - q)   LinkCell.cc:522
    ARITH_GHOST = 2, // r = g_j - q, g_j a stored copy (point or ghost)   CellIterator.h:173
};

// Cell-sorted view of a point set: points reordered by cell, with cell offsets.
struct DevGrid
{
    int dim[3];
    int ncell;
    const uint32_t* start; // ncell + 1 exclusive offsets
    const float4* cpos;    // positions sorted by cell; w = packed integer box image
    const uint32_t* cidx;  // original point index of each sorted slot
    // Ghost grid (ARITH_GHOST): axis-aligned cells of width 1 / ginv from gmin,
    // no wrap; a cell of position p is floor((p - gmin) * ginv) (CellQuery.h:53-59)
    int ghost = 0;
    float gmin[3] = {0.0f, 0.0f, 0.0f};
    float ginv = 0.0f;
};

// Ghost grid of a CellQuery (CellQuery.h:143-167, 218-299; CellQuery.cc:55-137):
// every point plus the ghost copies p + shift of points within r_cut (in
// fractional units fr) of a box face, on a padded axis-aligned grid.
struct GhostParams
{
    DevBox b;
    float fr[3];     // r_cut / nearest-plane distance, per axis
    float lat[3][3]; // lattice vectors (Box::getLatticeVector), lat[2] = 0 in 2D
    float gmin[3];
    float ginv;      // 1 / r_cut
    int dim[3];
};
// with_ghosts = 1: point grid (point + ghosts; copies outside the grid dropped).
// with_ghosts = 0: query grid (the point only; outside the grid -> bucket cell
// dim[0] * dim[1] * dim[2], which the kernels never visit).
// cell_count: ncell + 2 entries, zeroed. copy_cell / copy_rank: 8 per point.
void launch_ghost_count(const GhostParams& gp, const float* pts, uint32_t n, int with_ghosts, uint32_t* copy_cell,
                        uint32_t* copy_rank, uint32_t* cell_count, cudaStream_t s);
void launch_ghost_scatter(const GhostParams& gp, const float* pts, uint32_t n, int with_ghosts,
                          const uint32_t* copy_cell, const uint32_t* copy_rank, const uint32_t* start, float4* cpos,
                          uint32_t* cidx, cudaStream_t s);

// Per-query staging capacity of the warp-per-query emit kernel; queries with more
// bonds are written by the block-per-query kernel.
constexpr int EMIT_CAP = 256;
constexpr int HEAVY_CAP = 8192;

// ---- grid build ---------------------------------------------------------------
// Computes dims for a cell width and fills cell_of/rank and counts (atomics).
void launch_assign(const DevBox& box, const float* pts, uint32_t n, const int dim[3], uint32_t* cell_of,
                   uint32_t* rank, uint32_t* cell_count, cudaStream_t s);
void launch_scatter(const DevBox& box, const float* pts, uint32_t n, const uint32_t* cell_of,
                    const uint32_t* rank, const uint32_t* start, float4* cpos, uint32_t* cidx, cudaStream_t s);
// Every cell's points sorted by point index (cells of up to SORT_CELL_MAX points;
// larger cells stay in scatter order).
constexpr int SORT_CELL_MAX = 1024;
void launch_sort_cells(const uint32_t* start, int ncell, const float4* cpos_in, const uint32_t* cidx_in,
                       float4* cpos_out, uint32_t* cidx_out, cudaStream_t s);

// Exclusive scans. scratch must hold scan_scratch_bytes(n) bytes.
size_t scan_scratch_bytes(size_t n);
void scan_u32_to_u32(const uint32_t* in, uint32_t* out, size_t n, void* scratch, cudaStream_t s);
void scan_u32_to_u64(const uint32_t* in, uint64_t* out, size_t n, void* scratch, cudaStream_t s);

// ---- ball queries -------------------------------------------------------------
struct BallParams
{
    float r_max_sq;
    float r_min_sq;
    int exclude_ii;
    int arith;
    uint32_t nq;
};

// counts[i] = number of bonds of query i (original query index).
// list (optional): process only these positions of the sorted query array; p.nq is then the list length.
void launch_ball_count(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                       const BallParams& p, uint32_t* counts, cudaStream_t s, const uint32_t* list = nullptr);

// Writes bonds in reference order at offsets[i]. Queries with more than EMIT_CAP
// bonds are appended to heavy_list (heavy_count) and written by launch_ball_emit_heavy.
void launch_ball_emit(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                      const BallParams& p, const uint32_t* counts, const uint64_t* offsets, int by_distance,
                      uint2* ij, float* dist, float* vec, uint32_t* heavy_list, uint32_t* heavy_count,
                      int* err, cudaStream_t s, const uint32_t* list = nullptr);
void launch_ball_emit_heavy(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                            const BallParams& p, const uint32_t* counts, const uint64_t* offsets,
                            int by_distance, const uint32_t* heavy_list, uint32_t n_heavy, uint2* ij,
                            float* dist, float* vec, int* err, cudaStream_t s);

// Fused ball query + RDF histogram into uint64 counts (bins <= HIST_SMEM_BINS use
// block-private shared-memory histograms).
struct HistParams
{
    float h_min, h_max, h_inv;
    uint32_t bins;
    // optional exact r^2 -> bin table (frames histogram kernel): device words
    // [thresholds: bins + 2 floats][keys: u16], pairs counted iff rb_a <= r^2 < rb_b
    const uint32_t* rb = nullptr;
    uint32_t rb_words = 0;
    uint32_t rb_ut = 0; // bits of the first threshold above the first bin
    uint32_t rb_s = 0;  // key shift
    float rb_a = 0.0f, rb_b = 0.0f;
};
void launch_ball_hist(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                      const BallParams& p, const HistParams& h, unsigned long long* hist, cudaStream_t s,
                      const uint32_t* list = nullptr);

// Block-per-cell ball kernels. qg is the cell-sorted query grid (same dims as g).
// In the count pass, queries of cells whose candidate set exceeds CELL_CAP are
// appended to overflow for the warp-per-query kernels; the histogram pass tiles
// large candidate sets instead and never writes overflow (may be NULL there). pre_out2 > 0 enables the wrap-arithmetic
// prefilter (pairs beyond sqrt(pre_out2) are rejected without the exact test);
// pre_in2 > 0 lets the count pass accept pairs inside sqrt(pre_in2) unchecked.
// Scan pass (hist_mode 0): counts per query, acceptance masks gmask[nq][CELL_CHUNKS]
// (by sorted query position) and each cell's candidates sorted by point index,
// gsorted[ncell][CELL_CAP] (grid slot << 5 | wrap). hist_mode 1: fused histogram.
// Emit pass: writes each query's bonds, in (i, j) order, at offsets[i].
constexpr int CELL_CAP = 1024;
constexpr int CELL_CHUNKS = CELL_CAP / 32;
size_t cell_smem_bytes();
// n_points: number of points of g (point indices below 2^22 allow 32-bit merge keys).
// cull2 > 0 (count pass): candidates farther than sqrt(cull2) from the bounds of
// every query of the cell, in cell-shifted coordinates, are dropped before the
// merge; gtotal[cell] = candidates kept (all-ones for cells handed to the
// warp-per-query kernels), read by the emit pass.
// cap: candidate capacity of a cell in the count and emit passes, 1024 or 4096
// (dense point sets; cell_cap_for picks it); gsorted is [ncell][cap] and gmask
// [nq][cap / 32]. The histogram pass uses tiles of CELL_CAP.
int cell_cap_for(const DevGrid& g, uint32_t n_points, bool is2d);
void launch_cell_scan(int hist_mode, const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p,
                      float pre_out2, float pre_in2, float cull2, uint32_t* counts, uint32_t* gmask,
                      uint32_t* gsorted, uint32_t* gtotal, uint32_t* overflow, uint32_t* overflow_n,
                      const HistParams& h, unsigned long long* hist, cudaStream_t s,
                      uint32_t n_points = 0xffffffffu, int cap = CELL_CAP);
// Count pass with lanes over queries (same outputs as the count mode of
// launch_cell_scan, capacity CELL_CAP): wrap arithmetic with the prefilter on
// (pre_out2 > 0) and the per-cell cull (cull2 > 0) only.
void launch_nl_count(const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p, float pre_out2,
                     float pre_in2, float cull2, uint32_t* counts, uint32_t* gmask, uint32_t* gsorted,
                     uint32_t* gtotal, uint32_t* overflow, uint32_t* overflow_n, cudaStream_t s, uint32_t n_points);
void launch_cell_emit(const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p,
                      const uint32_t* gmask, const uint32_t* gsorted, const uint32_t* gtotal, const uint64_t* offsets,
                      uint2* ij, float* dist, float* vec, cudaStream_t s, int cap = CELL_CAP,
                      const uint32_t* counts = nullptr);

// Histogram of a distance array (RDF over a NeighborList).
void launch_hist_distances(const float* dist, uint64_t nb, const HistParams& h, unsigned long long* hist,
                           cudaStream_t s);

// CorrelationFunction over bonds (ij, distance): counts[bin] += 1 and
// sums[bin] += conj(values[j]) * qvalues[i] (FP64 complex as double2).
void launch_cf_bonds(const uint2* ij, const float* dist, uint64_t nb, const double2* values, const double2* qvalues,
                     const HistParams& h, double2* sums, unsigned long long* counts, cudaStream_t s);

// ---- PMFT ------------------------------------------------------------------------
enum PmftKind
{
    PMFT_R12 = 0,
    PMFT_XYT = 1,
    PMFT_XY = 2,
    PMFT_XYZ = 3,
};
// RegularAxis(n, min, max): inv = 1 / ((max - min) / n) in float (Histogram.h:126-131)
struct PmftAxis
{
    float min, max, inv;
    uint32_t n;
};
struct PmftParams
{
    PmftAxis ax[3];   // XY uses two
    uint32_t n_equiv; // XYZ equivalent orientations
};
// Bins every bond of a list: p_angle / q_angle per point / query (R12, XYT),
// q_cs = (cos, sin) of minus the query angle (XYT, XY), q_quat the query
// quaternions (s, x, y, z) and equiv the equivalent orientations (XYZ).
void launch_pmft_bonds(int kind, const uint2* ij, const float* dist, const float* vec, uint64_t nb,
                       const float* p_angle, const float* q_angle, const float2* q_cs, const float4* q_quat,
                       const float4* equiv, const PmftParams& pp, unsigned long long* hist, cudaStream_t s);

// ---- k nearest neighbours ------------------------------------------------------
struct KnnParams
{
    float r_max_sq;
    float r_min;     // AABB arithmetic filters on distance >= r_min
    float r_min_sq;  // wrap arithmetic filters on r_sq >= r_min^2
    int exclude_ii;
    int arith;
    uint32_t k;
    uint32_t nq;
    float covered;   // radius fully covered by the 27-cell stencil
};
// k <= 32: warp-per-query bitonic top-k over the 27-cell stencil. Results go to
// row i of (j, d, vec) temp arrays [nq * k]; counts[i] = number found. Queries
// whose k-th neighbour is not provably inside the stencil go to fail_list.
void launch_knn_warp(const DevBox& box, const DevGrid& g, const float4* qpos, const uint32_t* qidx,
                     const KnnParams& p, uint32_t* tj, float* td, float* tv, uint32_t* counts,
                     uint32_t* fail_list, uint32_t* fail_count, cudaStream_t s);
// Block-per-query brute force over every point (minimum over the 27 images in AABB
// arithmetic), used for k > 32 and for queries the warp kernel could not prove.
// list holds positions in the sorted query array. Any number of points; needs
// k <= knn_block_capacity() / 2 (else err = DEV_CAPACITY).
void launch_knn_block(const DevBox& box, const float4* cpos, const uint32_t* cidx, uint32_t n, const float4* qpos,
                      const uint32_t* qidx, const KnnParams& p, const uint32_t* list, uint32_t nlist, uint32_t* tj,
                      float* td, float* tv, uint32_t* counts, int* err, cudaStream_t s);
size_t knn_block_capacity();
// Compacts temp rows into a NeighborList (sorted by j, or by distance then j).
void launch_knn_compact(const uint32_t* tj, const float* td, const float* tv, uint32_t k, uint32_t nq,
                        const uint32_t* counts, const uint64_t* offsets, int by_distance, uint2* ij,
                        float* dist, float* vec, cudaStream_t s);

// ---- NeighborList helpers -------------------------------------------------------
void launch_fill_f32(float* a, float v, uint64_t n, cudaStream_t s);
// *flag |= 1 when a[0..n) and b[0..n) differ bitwise (flag zeroed by the caller).
void launch_words_differ(const uint32_t* a, const uint32_t* b, uint64_t n, uint32_t* flag, cudaStream_t s);
void launch_segments(const uint2* ij, uint64_t nb, uint32_t nq, uint32_t* segments, uint32_t* counts,
                     cudaStream_t s);
// segments[i] = counts[i] ? offsets[i] : 0 (NeighborList.cc:199-232 for a list built in query order)
void launch_segments_from_offsets(const uint32_t* counts, const uint64_t* offsets, uint32_t nq, uint32_t* segments,
                                  cudaStream_t s);

} // namespace fg
