/*
 * freud_gb300.h -- C ABI of the GB300-native neighbour-query -> pair-reduction
 * path (LinkCell / AABBQuery queries, NeighborList, RDF, Steinhardt).
 *
 * Every entry point returns an fg_status; on failure fg_last_error() gives a
 * thread-local message. Status classes mirror how the reference's C++ exceptions
 * reach Python (freud/locality/export-*.cc via nanobind):
 *   FG_ERR_VALUE   <- std::invalid_argument / std::domain_error  (ValueError)
 *   FG_ERR_RUNTIME <- std::runtime_error                         (RuntimeError)
 *   FG_ERR_INDEX   <- std::out_of_range                          (IndexError)
 *   FG_ERR_CUDA / FG_ERR_MEMORY for device failures               (RuntimeError)
 *
 * Host pointers are plain C arrays (float32 points are packed x,y,z triples, as
 * the reference's vec3<float>). Objects are opaque handles with explicit destroy.
 * Calls are synchronous: when a call returns, its results are complete.
 */
#ifndef FREUD_GB300_H
#define FREUD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int fg_status;
#define FG_OK 0
#define FG_ERR_VALUE 1
#define FG_ERR_RUNTIME 2
#define FG_ERR_INDEX 3
#define FG_ERR_CUDA 4
#define FG_ERR_MEMORY 5

/* Periodic box, freud::box::Box(Lx, Ly, Lz, xy, xz, yz, is2D)
 * (reference freud/box/Box.h:77-86; Python freud/box.py:58-76). */
typedef struct fg_box
{
    float Lx, Ly, Lz, xy, xz, yz;
    int is2D;
    int periodic_x, periodic_y, periodic_z;
} fg_box;

/* Query modes, freud::locality::QueryType (freud/locality/NeighborQuery.h:34-39). */
#define FG_MODE_NONE 0
#define FG_MODE_BALL 1
#define FG_MODE_NEAREST 2

/* freud::locality::QueryArgs (freud/locality/NeighborQuery.h:60-73), same defaults:
 * num_neighbors 0xffffffff, r_max -1, r_min 0, r_guess -1, scale -1, exclude_ii 0. */
typedef struct fg_query_args
{
    int mode;
    uint32_t num_neighbors;
    float r_max;
    float r_min;
    float r_guess;
    float scale;
    int exclude_ii;
} fg_query_args;

/* Neighbour-query kinds. RAWPOINTS is the reference's default behind every
 * (box, points) tuple (freud/locality/RawPoints.h:30-77) and uses AABB arithmetic. */
#define FG_NQ_RAWPOINTS 0
#define FG_NQ_AABB 1
#define FG_NQ_LINKCELL 2
#define FG_NQ_CELLQUERY 3 /* freud::locality::CellQuery (CellQuery.h:30-318): ball queries only */

typedef struct fg_nq fg_nq;
typedef struct fg_nlist fg_nlist;
typedef struct fg_rdf fg_rdf;
typedef struct fg_cf fg_cf;
typedef struct fg_pmft fg_pmft;
typedef struct fg_steinhardt fg_steinhardt;
typedef struct fg_frames fg_frames;

/* Library */
const char* fg_last_error(void);
int fg_version(void);
/* Stream the library launches on (a cudaStream_t); NULL restores the library's own. */
fg_status fg_set_stream(void* cuda_stream);

/* Kernel launch accounting and per-kernel device timing (no counterpart in the
 * reference, which has no device code). fg_launch_count: kernels launched by
 * this library since load. fg_profile_enable(1) resets the per-kernel table and
 * brackets every launch with CUDA events on its stream; fg_profile_report writes
 * one line "name launches total_ms" per kernel. */
fg_status fg_launch_count(uint64_t* out);
fg_status fg_profile_enable(int enable);
fg_status fg_profile_report(char* buf, size_t len);

/* ---- NeighborQuery -------------------------------------------------------
 * Replaces freud::locality::AABBQuery(box, points, n) (freud/locality/AABBQuery.cc:18-24),
 * LinkCell(box, points, n, cell_width) (freud/locality/LinkCell.cc:222-260) and
 * RawPoints(box, points, n) (freud/locality/RawPoints.h:36-38); Python bindings
 * freud/locality/export-NeighborQuery.cc:35-65. Points are copied to the device. */
fg_status fg_nq_create(const fg_box* box, const float* points, uint32_t n, int kind, float cell_width, fg_nq** out);
/* Same with points already resident on the current device (not copied, must outlive the handle). */
fg_status fg_nq_create_device(const fg_box* box, const float* device_points, uint32_t n, int kind, float cell_width,
                              fg_nq** out);
fg_status fg_nq_destroy(fg_nq* nq);
/* LinkCell::getCellWidth (freud/locality/LinkCell.h:189-192). */
fg_status fg_nq_cell_width(const fg_nq* nq, float* out);
fg_status fg_nq_num_points(const fg_nq* nq, uint32_t* out);
/* NeighborQuery::getPoints (NeighborQuery.h:145-153): the object's points (n x 3
 * float32, as they were given) copied to out. */
fg_status fg_nq_get_points(const fg_nq* nq, float* out);

/* NeighborQuery::query(...) -> NeighborQueryIterator::toNeighborList(sort_by_distance)
 * (freud/locality/NeighborQuery.h:130-142, 434-481; export-NeighborQuery.cc:26-33,130-135).
 * query_points == NULL queries the object's own points. Bonds come out in the
 * reference order: (i, j, weight, distance), or (i, distance, j, weight). Host
 * query points are copied on a second stream the library owns while the object's
 * cell grid is built; the call returns after the copy and the query are done, so
 * the caller may release query_points then. */
fg_status fg_nq_query(fg_nq* nq, const float* query_points, uint32_t n_query, const fg_query_args* args,
                      int sort_by_distance, fg_nlist** out);
/* Same with query points already on the device. */
fg_status fg_nq_query_device(fg_nq* nq, const float* device_query_points, uint32_t n_query,
                             const fg_query_args* args, int sort_by_distance, fg_nlist** out);

/* ---- NeighborList ----------------------------------------------------------
 * freud::locality::NeighborList (freud/locality/NeighborList.h:29-158, .cc:24-430;
 * bindings freud/locality/export-NeighborList.cc:24-86). */
/* NeighborList(num_bonds, query_point_index, num_query_points, point_index, num_points,
 * vectors, weights) (NeighborList.cc:51-82): validates sorted query indices; distances
 * are sqrt(dot(v, v)). weights may be NULL (all 1). */
fg_status fg_nlist_from_arrays(uint64_t num_bonds, const uint32_t* query_point_indices, uint32_t num_query_points,
                               const uint32_t* point_indices, uint32_t num_points, const float* vectors,
                               const float* weights, fg_nlist** out);
/* NeighborList(points, query_points, box, exclude_ii) all pairs (NeighborList.cc:84-128). */
fg_status fg_nlist_all_pairs(const fg_box* box, const float* points, uint32_t num_points, const float* query_points,
                             uint32_t num_query_points, int exclude_ii, fg_nlist** out);
fg_status fg_nlist_destroy(fg_nlist* nl);
/* NeighborList::copy (NeighborList.cc:354-366). */
fg_status fg_nlist_copy(const fg_nlist* src, fg_nlist** out);
fg_status fg_nlist_num_bonds(const fg_nlist* nl, uint64_t* out);
fg_status fg_nlist_num_query_points(const fg_nlist* nl, uint32_t* out);
fg_status fg_nlist_num_points(const fg_nlist* nl, uint32_t* out);
/* getNeighbors (B,2) / getDistances / getWeights / getVectors (B,3) copied to host;
 * any output may be NULL. */
fg_status fg_nlist_get(const fg_nlist* nl, uint32_t* neighbors, float* distances, float* weights, float* vectors);
/* Device pointers of the bond arrays (valid until the list is destroyed or modified). */
/* Page-locked host memory (cudaMallocHost / cudaFreeHost), no reference counterpart:
 * the Python layer returns large NeighborList arrays in such buffers (pooled), so
 * fg_nlist_get copies them from the device by DMA at the link's rate instead of
 * through the driver's staging of pageable memory. */
fg_status fg_host_alloc(size_t bytes, void** out);
fg_status fg_host_free(void* p);

fg_status fg_nlist_device_arrays(const fg_nlist* nl, const uint32_t** neighbors, const float** distances,
                                 const float** vectors);
/* getSegments / getCounts (NeighborList.cc:199-232). */
fg_status fg_nlist_segments(const fg_nlist* nl, uint32_t* segments, uint32_t* counts);
/* find_first_index (NeighborList.cc:309-316). */
fg_status fg_nlist_find_first_index(const fg_nlist* nl, uint32_t i, uint32_t* out);
/* filter(bool*) (NeighborList.cc:234-284); keep is one byte per bond. */
fg_status fg_nlist_filter(fg_nlist* nl, const uint8_t* keep);
/* filter_r (NeighborList.cc:286-307). */
fg_status fg_nlist_filter_r(fg_nlist* nl, float r_max, float r_min);
/* sort(by_distance) (NeighborList.cc:371-399). */
fg_status fg_nlist_sort(fg_nlist* nl, int by_distance);

/* ---- RDF ---------------------------------------------------------------------
 * freud::density::RDF (freud/density/RDF.cc:25-110; bindings export-RDF.cc:22-47,
 * BondHistogramCompute export-BondHistogramCompute.cc:67-76). */
fg_status fg_rdf_create(uint32_t bins, float r_max, float r_min, fg_rdf** out);
fg_status fg_rdf_destroy(fg_rdf* rdf);
/* RDF::mode: 0 = exact, 1 = finite_size (RDF.h:20-24). */
fg_status fg_rdf_set_mode(fg_rdf* rdf, int finite_size);
/* BondHistogramCompute::reset (BondHistogramCompute.h:39-49). */
fg_status fg_rdf_reset(fg_rdf* rdf);
/* RDF::accumulate (RDF.cc:101-110): nlist == NULL queries nq with args. */
fg_status fg_rdf_accumulate(fg_rdf* rdf, fg_nq* nq, const float* query_points, uint32_t n_query,
                            const fg_nlist* nlist, const fg_query_args* args);
/* Same with query points already on the device. */
fg_status fg_rdf_accumulate_device(fg_rdf* rdf, fg_nq* nq, const float* device_query_points, uint32_t n_query,
                                   const fg_nlist* nlist, const fg_query_args* args);
/* getBinCounts (uint32, reference dtype), getRDF, getNr (RDF.cc:73-99, float32 arithmetic
 * identical to the reference). Any output may be NULL. */
fg_status fg_rdf_get(fg_rdf* rdf, uint32_t* bin_counts, float* rdf_out, float* n_r);
/* Full-width uint64 counts and an FP64 normalisation of the same quantities. */
fg_status fg_rdf_get_u64(fg_rdf* rdf, uint64_t* bin_counts, double* rdf_out, double* n_r);
/* getBinEdges / getBinCenters (Histogram.h:72-80, 126-138). */
fg_status fg_rdf_bin_edges(const fg_rdf* rdf, float* edges, float* centers);
/* getBox of the last accumulated frame; frame counter. */
fg_status fg_rdf_state(const fg_rdf* rdf, fg_box* box, uint32_t* n_frames, uint32_t* n_points, uint32_t* n_query);
/* No counterpart in the reference: replaces the accumulated state (uint64 bin
 * counts, frame counter, last frame's box and N) - used to load the combination
 * of RDFs accumulated over disjoint frame ranges by several processes (one GPU
 * each), so rdf / n_r come out as if one process had accumulated every frame. */
fg_status fg_rdf_set_state(fg_rdf* rdf, const uint64_t* bin_counts, uint32_t n_frames, const fg_box* box,
                           uint32_t n_points, uint32_t n_query);

/* ---- CorrelationFunction ----------------------------------------------------------
 * freud::density::CorrelationFunction (freud/density/CorrelationFunction.cc:26-99;
 * bindings export-CorrelationFunction.cc; Python freud/density.py:28-177). Values are
 * complex double (re, im interleaved), as the reference converts them. */
fg_status fg_cf_create(uint32_t bins, float r_max, fg_cf** out);
fg_status fg_cf_destroy(fg_cf* cf);
/* BondHistogramCompute::reset + the correlation sums (CorrelationFunction.cc:61-66). */
fg_status fg_cf_reset(fg_cf* cf);
/* CorrelationFunction::accumulate (CorrelationFunction.cc:79-96): for every bond
 * (query i, point j), bin its distance and add conj(values[j]) * query_values[i].
 * n_values must equal the number of points; query_values == NULL uses values;
 * nlist == NULL queries nq with args. */
fg_status fg_cf_accumulate(fg_cf* cf, fg_nq* nq, const double* values, uint32_t n_values,
                           const float* query_points, uint32_t n_query, const double* query_values,
                           uint32_t n_query_values, const fg_nlist* nlist, const fg_query_args* args);
/* getBinCounts (uint32) and getCorrelation (sum / count per bin where the count is
 * nonzero, CorrelationFunction.cc:48-59; complex double interleaved). Either may be NULL. */
fg_status fg_cf_get(fg_cf* cf, uint32_t* bin_counts, double* correlation);
/* getBinEdges / getBinCenters (Histogram.h:72-80, 126-138). */
fg_status fg_cf_bin_edges(const fg_cf* cf, float* edges, float* centers);
/* getBox of the last accumulated frame; frame counter. */
fg_status fg_cf_state(const fg_cf* cf, fg_box* box, uint32_t* n_frames);

/* ---- PMFT -------------------------------------------------------------------------
 * freud::pmft::PMFTR12 / PMFTXYT / PMFTXY / PMFTXYZ (freud/pmft/PMFTR12.cc, PMFTXYT.cc,
 * PMFTXY.cc, PMFTXYZ.cc, PMFT.h:29-88;
 * bindings freud/pmft/export-PMFT*; Python freud/pmft.py). */
#define FG_PMFT_R12 0 /* maxes = {r_max}, bins = {n_r, n_t1, n_t2} */
#define FG_PMFT_XYT 1 /* maxes = {x_max, y_max}, bins = {n_x, n_y, n_t} */
#define FG_PMFT_XY 2  /* maxes = {x_max, y_max}, bins = {n_x, n_y} */
#define FG_PMFT_XYZ 3 /* maxes = {x_max, y_max, z_max}, bins = {n_x, n_y, n_z} */
fg_status fg_pmft_create(int kind, const float* maxes, const uint32_t* bins, fg_pmft** out);
fg_status fg_pmft_destroy(fg_pmft* pm);
fg_status fg_pmft_reset(fg_pmft* pm);
/* PMFT*::accumulate: orientations are per-point angles (R12, XYT; NULL otherwise),
 * query_orientations per-query angles (R12, XYT, XY; NULL: orientations for R12 /
 * XYT) or quaternions (s, x, y, z) (XYZ); equiv_orientations quaternions (XYZ).
 * nlist == NULL queries nq with args. */
fg_status fg_pmft_accumulate(fg_pmft* pm, fg_nq* nq, const float* orientations, uint32_t n_orient,
                             const float* query_points, uint32_t n_query, const float* query_orientations,
                             uint32_t n_query_orient, const float* equiv_orientations, uint32_t n_equiv,
                             const fg_nlist* nlist, const fg_query_args* args);
/* getBinCounts (uint32, row-major over the axes) and getPCF (PMFT.h:70-82). */
fg_status fg_pmft_get(fg_pmft* pm, uint32_t* bin_counts, float* pcf);
/* One axis: bin edges (n + 1), centres (n), bounds (min, max), bin count. */
fg_status fg_pmft_axis(const fg_pmft* pm, int axis, float* edges, float* centers, float* bounds, uint32_t* n);
/* getBox of the last accumulated frame; frame counter. */
fg_status fg_pmft_state(const fg_pmft* pm, fg_box* box, uint32_t* n_frames);

/* ---- Steinhardt ----------------------------------------------------------------
 * freud::order::Steinhardt (freud/order/Steinhardt.h:59-223, Steinhardt.cc:85-359;
 * bindings export-Steinhardt.cc:19-34). */
fg_status fg_steinhardt_create(const uint32_t* ls, uint32_t n_l, int average, int wl, int weighted,
                               int wl_normalize, fg_steinhardt** out);
fg_status fg_steinhardt_destroy(fg_steinhardt* st);
/* Steinhardt::compute(nlist, points, qargs): nlist == NULL queries nq with args. */
fg_status fg_steinhardt_compute(fg_steinhardt* st, fg_nq* nq, const fg_nlist* nlist, const fg_query_args* args);
fg_status fg_steinhardt_num_particles(const fg_steinhardt* st, uint32_t* out);
/* getQl (N, n_l), getParticleOrder (N, n_l), getQlm (per l an (N, 2l+1) complex64
 * array, concatenated in l order, as interleaved re/im floats), getOrder (n_l).
 * Any output may be NULL. */
fg_status fg_steinhardt_get(const fg_steinhardt* st, float* ql, float* particle_order, float* qlm, float* order);

/* ---- Allocation-free RDF histogram -----------------------------------------
 * No counterpart in the reference (freud has no device code). For callers that
 * may not allocate device memory - an analysis plugin inside a simulation engine
 * that owns every device allocation, or code under an allocator that forbids
 * cudaMalloc - this computes the uint64 RDF bin counts of one frame (the ball
 * query of radius r_max with bins over [r_min, r_max), as
 * RDF(bins, r_max, r_min).compute((box, points)) does, fused) without allocating
 * anything: its scratch is a fixed file-scope device array of 4,203,520 bytes that
 * every GPU loading the library holds until exit, which limits n to 65,536 points
 * (larger n is rejected with FG_ERR_VALUE). device_points (n x 3 float32) and
 * device_counts (bins uint64, overwritten) are the caller's device buffers.
 * kind: FG_NQ_RAWPOINTS / FG_NQ_AABB (AABB arithmetic) or FG_NQ_LINKCELL (wrap).
 * Work is enqueued on cuda_stream (NULL: the legacy default stream) and the call
 * returns without synchronising. The first call on each device looks up the
 * scratch array's device address, so make it before any stream capture. All
 * calls share the scratch: calls that overlap on the GPU race. */
fg_status fg_rdf_histogram_noalloc(const fg_box* box, const float* device_points, uint32_t n, float r_max,
                                   float r_min, uint32_t bins, int exclude_ii, int kind,
                                   unsigned long long* device_counts, void* cuda_stream);

/* ---- Batched frames ----------------------------------------------------------
 * No single counterpart in the reference: a batch stands for a sequence of
 * (box, points) systems (RawPoints, NeighborQuery.h / RawPoints.h:30-77) that a
 * freud user passes one per compute call, e.g. RDF.compute(system, reset=False)
 * over a trajectory (BondHistogramCompute.h:115-126). The batch holds F frames of
 * uneven N on the device; points are concatenated frame after frame
 * (frame_offsets: F + 1 ascending point offsets, offsets[0] = 0, every frame
 * non-empty) and point indices in every per-point output are global (into the
 * concatenation). boxes: F periodic boxes. Pair arithmetic is AABB arithmetic
 * (AABBQuery.cc:93,125), as for a (box, points) system. */
fg_status fg_frames_create(const fg_box* boxes, const float* points, const uint64_t* frame_offsets, uint32_t n_frames,
                           fg_frames** out);
/* As fg_frames_create with one host array per frame (frame_points[f]: n_f x 3
 * float32), copied straight into the batch's device buffer. */
fg_status fg_frames_create_list(const fg_box* boxes, const float* const* frame_points, const uint64_t* frame_offsets,
                                uint32_t n_frames, fg_frames** out);
/* As fg_frames_create with the caller's device points (borrowed, not copied). */
fg_status fg_frames_create_device(const fg_box* boxes, const float* device_points, const uint64_t* frame_offsets,
                                  uint32_t n_frames, fg_frames** out);
/* New positions for a batch created from host points (same frames and N). */
fg_status fg_frames_set_points(fg_frames* frames, const float* points);
fg_status fg_frames_destroy(fg_frames* frames);
fg_status fg_frames_info(const fg_frames* frames, uint32_t* n_frames, uint64_t* n_points);
/* Same result as F calls of RDF::accumulate (RDF.cc:101-110) with a ball query
 * (args: mode ball, r_max, r_min, exclude_ii) on each frame in order: bin counts
 * summed, frame counter += F, box and N of the last frame. */
fg_status fg_rdf_accumulate_frames(fg_rdf* rdf, fg_frames* frames, const fg_query_args* args);
/* Steinhardt::compute (Steinhardt.cc:85-118) of every frame with its own ball
 * query (args as above). Per-particle outputs (fg_steinhardt_get) cover all
 * points in batch order; the order output holds n_frames x n_l values. */
fg_status fg_steinhardt_compute_frames(fg_steinhardt* st, fg_frames* frames, const fg_query_args* args);
/* Frames covered by the last compute (1 after fg_steinhardt_compute). */
fg_status fg_steinhardt_num_frames(const fg_steinhardt* st, uint32_t* out);
/* Launch shape of the batched RDF kernel: shell 1 (27 cells of width >= r_max)
 * or 2 (125 cells of width >= r_max / 2), 4 or 8 warps per block, 1 or 2
 * privatised shared histograms per block. shell 0 (default) = autotuned: the
 * candidates are timed on the first batch of each kind and the fastest is kept. */
fg_status fg_batch_set_config(int shell, int warps_per_block, int hist_copies);
/* Count pass of ball-query NeighborLists: 0 (default) picks the lanes-over-queries
 * kernel where it applies (LinkCell arithmetic with the cell-shift prefilter,
 * stencils of at most 1024 candidates after the cull) and the block-per-cell
 * lanes-over-candidates kernel elsewhere; 1 always takes the latter. Both give
 * the same list; the switch exists to compare them. */
fg_status fg_set_count_kernel(int which);
/* Text log of the autotuner's measurements and choices. */
fg_status fg_autotune_report(char* buf, size_t len);
/* Batched calls record their device work as CUDA graphs and replay them (1,
 * default) or launch it directly (0). */
fg_status fg_set_graphs(int enable);

/* Self-check of the device division that the box arithmetic uses (no counterpart
 * in the reference, whose Box::makeFractional, Box.h:243-255, divides with the
 * host's IEEE division): the quotients of `samples` seeded (a, b) pairs (box
 * lengths and random divisors, dividends of either sign) computed from a
 * precomputed reciprocal are compared bit for bit with CUDA's IEEE division;
 * *mismatches receives the number that differ and example (optional, 2 floats)
 * one differing (a, b). Synchronous. */
fg_status fg_check_division(uint64_t samples, uint64_t seed, uint64_t* mismatches, float* example);

#ifdef __cplusplus
}
#endif

#endif /* FREUD_GB300_H */
