// Launch interface of the batched (many frames, one launch) kernels.
//
// A batch holds F frames of uneven N: points concatenated frame after frame,
// each frame with its own periodic box. One cell grid spans every frame: frame
// f owns the cells [cell_base[f], cell_base[f + 1]) and the points
// [pt_base[f], pt_base[f + 1]); point indices are global (into the
// concatenation), so per-point outputs of every frame land in one array.
// Pair arithmetic is the AABB arithmetic of a (box, points) system
// (AABBQuery.cc:93,125): r = p_j - (q + image_k), k = n_j - n_q - wrap.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "fg_kernels.cuh"
#include "fg_steinhardt.cuh"

namespace fg {

struct FrameDesc
{
    DevBox b;
    int dim[3];
    int shell;          // stencil half-width in cells: cells are >= r_max / shell wide
    uint32_t cell_base; // first cell of the frame in the batch grid
    uint32_t ncell;
    uint32_t pt_base;   // first point of the frame
    uint32_t n;
};

// Cell grid over every frame of a batch.
struct BatchGrid
{
    const FrameDesc* fd;       // [nframes]
    const uint32_t* cell_base; // [nframes + 1]
    uint32_t nframes;
    uint32_t ncell;            // all frames
    const uint32_t* start;     // [ncell + 1] exclusive offsets into the point slots
    const float4* cpos;        // cell-sorted positions, w = packed integer box image
    const uint32_t* cidx;      // global point index of each slot
    const uint32_t* cell_of;   // global cell of each point (by point index)
    const int* frame_out;      // [nframes]: nonzero when some point of the frame lies outside its box
};

// Tunable launch shape of the batched histogram kernel.
struct BatchHistConfig
{
    int shell;  // 1: 27-cell stencil of r_max cells; 2: 125-cell stencil of r_max / 2 cells
    int warps;  // warps per block (4 or 8)
    int copies; // privatised shared histograms per block (1 or 2)
};

// Counting sort of every frame's points into the batch grid. cell_count must be
// zeroed ([ncell + 1]); pos4 receives (x, y, z, image) per point.
// frame_out ([nframes], zeroed) is set for each frame with a point outside its box.
void launch_frames_assign(const FrameDesc* fd, const uint32_t* pt_base, uint32_t nframes, const float* pts,
                          uint32_t n, uint32_t* cell_of, uint32_t* rank, float4* pos4, uint32_t* cell_count,
                          int* frame_out, cudaStream_t s);
void launch_frames_scatter(uint32_t n, const uint32_t* cell_of, const uint32_t* rank, const float4* pos4,
                           const uint32_t* start, float4* cpos, uint32_t* cidx, cudaStream_t s);

// Fused ball query + RDF histogram over every cell of the batch: persistent
// blocks pull runs of cells from a device work counter (*queue, zeroed before
// the launch) until cell_limit. hist is uint64[h.bins]. With exclude_ii, frames
// whose points all lie in the box count each unordered pair once (half stencil;
// see k_frames_hist).
size_t frames_hist_smem_bytes();

// h with its exact r^2 -> bin table filled in (the pair test r_min_sq <= r^2 <
// r_max_sq folded in), or h unchanged when the table does not fit the kernel's
// shared memory. Tables are built once per parameter set and kept for the life of
// the process, so graphs may hold their pointers; call outside stream capture.
HistParams with_rsq_bins(const HistParams& h, float r_min_sq, float r_max_sq);
void launch_frames_hist(const BatchHistConfig& cfg, const BatchGrid& g, const BallParams& p, const HistParams& h,
                        uint32_t cell_limit, uint32_t* queue, unsigned long long* hist, cudaStream_t s);

// Ball query over every frame (grid of r_max cells, shell 1), warp per cell.
// Count pass: counts[i] = bonds of point i. Fill pass: bonds of point i at
// offsets[i] in candidate order: the neighbour index j and one float4 holding the
// Steinhardt bond vector box.wrap(p_j - p_i) (Steinhardt.cc:155) and the distance.
void launch_frames_ball_count(const BatchGrid& g, const BallParams& p, uint32_t n, uint32_t* counts, cudaStream_t s);
void launch_frames_ball_fill(const BatchGrid& g, const BallParams& p, uint32_t n, const uint64_t* offsets,
                             uint32_t* bond_j, float4* bond_vd, cudaStream_t s);
// One pass without the counts: warps take chunks of the bond arrays (capacity
// cap) from *alloc (zeroed before the launch); seg[i] / counts[i] = the first bond
// of point i and its bond count, its bonds in candidate order. *alloc > cap after
// the launch: the arrays were too small and nothing past cap was written.
uint64_t frames_ball_onepass_slack(uint32_t ncell); // bond slots the chunk tails may leave unused
void launch_frames_ball_onepass(const BatchGrid& g, const BallParams& p, uint32_t n, uint32_t* counts, uint32_t* seg,
                                uint32_t* bond_j, float4* bond_vd, unsigned long long* alloc, uint64_t cap,
                                cudaStream_t s);

// Per-frame FP64 system sums of the per-l (n, 2l + 1) qlm layout: sys[f][col]
// (complex, col running over every l's m) = (FP64 sum over the frame's rows) /
// n_f: float-float (exact TwoSum) running sums over runs of at most FRAME_SYS_ROWS
// rows, FP64 from there on (fixed shuffle trees, then a fixed tree over the runs),
// so results do not depend on scheduling. max_rows is the
// largest frame; partial holds nframes * frames_sys_splits(max_rows) * stride * 2
// doubles.
constexpr uint32_t FRAME_SYS_ROWS = 512;
int frames_sys_splits(uint32_t max_rows);
void launch_frames_sys(const uint32_t* pt_base, uint32_t nframes, uint32_t max_rows, const StLs& ls, int stride,
                       const float2* src, double* partial, double* sys, cudaStream_t s);

} // namespace fg
