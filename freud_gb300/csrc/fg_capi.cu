// Host runtime and C ABI of freud_gb300 (declared in include/freud_gb300.h).
//
// Mirrors the reference's object model (NeighborQuery / NeighborList / RDF /
// Steinhardt, freud/locality, freud/density, freud/order) over device-resident
// buffers. Argument validation and error classes follow the reference's C++
// (NeighborQuery.h:86-111, 195-228, 315-329, 496-509; LinkCell.cc:222-260;
// RDF.cc:25-42; NeighborList.cc:51-82, 286-307). All device work is issued on one
// stream; every entry point synchronises before returning.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/freud_gb300.h"
#include "fg_batch.cuh"
#include "fg_kernels.cuh"
#include "fg_nlist.cuh"
#include "fg_prof.cuh"
#include "fg_steinhardt.cuh"

namespace fg {

// ---------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------
struct Error : std::runtime_error
{
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};
static thread_local std::string g_last_error;

#define FG_CUDA(call)                                                                                            \
    do                                                                                                           \
    {                                                                                                            \
        cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess)                                                                                   \
        {                                                                                                        \
            throw Error(e_ == cudaErrorMemoryAllocation ? FG_ERR_MEMORY : FG_ERR_CUDA,                           \
                        std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #call);                    \
        }                                                                                                        \
    } while (0)

static void value_error(const std::string& m)
{
    throw Error(FG_ERR_VALUE, m);
}
static void runtime_error(const std::string& m)
{
    throw Error(FG_ERR_RUNTIME, m);
}
static void index_error(const std::string& m)
{
    throw Error(FG_ERR_INDEX, m);
}

// ---------------------------------------------------------------------------
// Stream and device memory
// ---------------------------------------------------------------------------
static cudaStream_t g_user_stream = nullptr;
static bool g_user_stream_set = false;

static void keep_pool(int dev)
{
    // keep freed blocks in the stream-ordered pool for reuse across frames
    static bool done[64] = {false};
    if (dev >= 0 && dev < 64 && !done[dev])
    {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
        {
            uint64_t thr = std::numeric_limits<uint64_t>::max();
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
        done[dev] = true;
    }
}

static cudaStream_t stream()
{
    if (g_user_stream_set)
    {
        int dev = 0;
        if (cudaGetDevice(&dev) == cudaSuccess)
            keep_pool(dev);
        return g_user_stream;
    }
    static thread_local cudaStream_t own = nullptr;
    static thread_local int own_dev = -1;
    int dev = 0;
    FG_CUDA(cudaGetDevice(&dev));
    if (own == nullptr || own_dev != dev)
    {
        FG_CUDA(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        own_dev = dev;
        keep_pool(dev);
    }
    return own;
}

// Stream-ordered device buffer.
struct DevBuf
{
    void* p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes)
    {
        o.p = nullptr;
        o.bytes = 0;
    }
    DevBuf& operator=(DevBuf&& o) noexcept
    {
        if (this != &o)
        {
            release();
            p = o.p;
            bytes = o.bytes;
            o.p = nullptr;
            o.bytes = 0;
        }
        return *this;
    }
    ~DevBuf() { release(); }
    void release()
    {
        if (p != nullptr)
        {
            cudaFreeAsync(p, stream());
            p = nullptr;
            bytes = 0;
        }
    }
    void alloc(size_t n)
    {
        if (n <= bytes && p != nullptr)
        {
            return;
        }
        release();
        const size_t want = n == 0 ? 16 : n;
        FG_CUDA(cudaMallocAsync(&p, want, stream()));
        bytes = want;
    }
    template<typename T> T* as() const { return static_cast<T*>(p); }
};

static void sync()
{
    FG_CUDA(cudaStreamSynchronize(stream()));
    FG_CUDA(cudaGetLastError());
}

// Device error word shared by the kernels of one call.
static int* dev_err()
{
    static thread_local DevBuf* buf = nullptr;
    if (buf == nullptr)
    {
        buf = new DevBuf();
        buf->alloc(sizeof(int));
    }
    return buf->as<int>();
}

static void reset_dev_err()
{
    FG_CUDA(cudaMemsetAsync(dev_err(), 0, sizeof(int), stream()));
}

static void check_dev_err(const char* what)
{
    int h = 0;
    FG_CUDA(cudaMemcpyAsync(&h, dev_err(), sizeof(int), cudaMemcpyDeviceToHost, stream()));
    sync();
    if (h == DEV_CAPACITY)
    {
        runtime_error(std::string(what) + ": a per-query capacity limit was exceeded");
    }
    if (h != DEV_OK)
    {
        runtime_error(std::string(what) + ": device error code " + std::to_string(h));
    }
}

// ---------------------------------------------------------------------------
// Box (host float32 arithmetic in the reference order; built with -ffp-contract=off)
// ---------------------------------------------------------------------------
struct HostBox
{
    float L[3];
    float xy, xz, yz;
    bool is2d;
    bool periodic[3];
};

static HostBox to_host_box(const fg_box* b)
{
    HostBox h;
    h.is2d = b->is2D != 0;
    h.L[0] = b->Lx;
    h.L[1] = b->Ly;
    h.L[2] = h.is2d ? 0.0f : b->Lz;
    h.xy = b->xy;
    h.xz = b->xz;
    h.yz = b->yz;
    h.periodic[0] = b->periodic_x != 0;
    h.periodic[1] = b->periodic_y != 0;
    h.periodic[2] = b->periodic_z != 0;
    return h;
}

static fg_box to_c_box(const HostBox& h)
{
    fg_box b;
    b.Lx = h.L[0];
    b.Ly = h.L[1];
    b.Lz = h.L[2];
    b.xy = h.xy;
    b.xz = h.xz;
    b.yz = h.yz;
    b.is2D = h.is2d ? 1 : 0;
    b.periodic_x = h.periodic[0];
    b.periodic_y = h.periodic[1];
    b.periodic_z = h.periodic[2];
    return b;
}

// Box::getNearestPlaneDistance, Box.h:489-497
static void nearest_plane(const HostBox& b, float d[3])
{
    const float t = fsub(fmul(b.xy, b.yz), b.xz);
    d[0] = fdiv(b.L[0], std::sqrt(fadd(fadd(1.0f, fmul(b.xy, b.xy)), fmul(t, t))));
    d[1] = fdiv(b.L[1], std::sqrt(fadd(1.0f, fmul(b.yz, b.yz))));
    d[2] = b.L[2];
}

static float box_volume(const HostBox& b)
{
    return b.is2d ? fmul(b.L[0], b.L[1]) : fmul(fmul(b.L[0], b.L[1]), b.L[2]);
}

// DevBox with the reference's image vectors (NeighborQuery.h:531-560):
// image(i, j, k) = (float(i) * a1 + float(j) * a2) + float(k) * a3.
static DevBox make_devbox(const HostBox& h)
{
    DevBox d;
    for (int a = 0; a < 3; ++a)
    {
        d.L[a] = h.L[a];
        d.lo[a] = -(fdiv(h.L[a], 2.0f));
    }
    d.xy = h.xy;
    d.xz = h.xz;
    d.yz = h.yz;
    d.is2d = h.is2d ? 1 : 0;
    for (int a = 0; a < 3; ++a)
        d.rcp[a] = h.L[a] != 0.0f ? fdiv(1.0f, h.L[a]) : 0.0f;
    d.tilted = (h.xy != 0.0f || h.xz != 0.0f || h.yz != 0.0f) ? 1 : 0;
    const float a1[3] = {h.L[0], 0.0f, 0.0f};
    const float a2[3] = {fmul(h.L[1], h.xy), h.L[1], 0.0f};
    float a3[3] = {0.0f, 0.0f, 0.0f};
    if (!h.is2d)
    {
        a3[0] = fmul(h.L[2], h.xz);
        a3[1] = fmul(h.L[2], h.yz);
        a3[2] = h.L[2];
    }
    for (int i = -1; i <= 1; ++i)
    {
        for (int j = -1; j <= 1; ++j)
        {
            for (int k = -1; k <= 1; ++k)
            {
                const int code = (i + 1) * 9 + (j + 1) * 3 + (k + 1);
                for (int c = 0; c < 3; ++c)
                {
                    d.img[code][c] = fadd(fadd(fmul(static_cast<float>(i), a1[c]), fmul(static_cast<float>(j), a2[c])),
                                          fmul(static_cast<float>(k), a3[c]));
                }
            }
        }
    }
    return d;
}

} // namespace fg

using namespace fg;

// ---------------------------------------------------------------------------
// Opaque handles
// ---------------------------------------------------------------------------
struct GridEntry
{
    int dim[3];
    int ncell;
    DevBuf start, cpos, cidx;
    // ghost grid of a CellQuery (r_cut = the query's r_max)
    bool ghost = false;
    float r_cut = 0.0f;
    GhostParams gp {};
};

struct fg_nq
{
    HostBox box;
    DevBox dbox;
    int kind;
    float cell_width;
    uint32_t n;
    const float* dpts;
    DevBuf own;
    std::vector<std::unique_ptr<GridEntry>> grids;
    std::vector<std::unique_ptr<GridEntry>> ghost_grids; // CellQuery, per r_cut
};

struct fg_nlist
{
    uint64_t nb = 0;
    uint32_t nq = 0, np = 0;
    DevBuf ij, dist, vec, weights; // weights empty => all 1
    bool unit_weights = true;
    DevBuf seg, cnt;
    bool seg_valid = false;
};

struct fg_rdf
{
    uint32_t bins;
    float r_max, r_min;
    int finite_size = 0;
    DevBuf hist;
    HostBox box {};
    uint32_t frames = 0, n_points = 0, n_query = 0;
};

struct fg_cf
{
    uint32_t bins;
    float r_max;
    DevBuf sums;   // double2 per bin: running sum of conj(values[j]) * query_values[i]
    DevBuf counts; // uint64 per bin
    HostBox box {};
    uint32_t frames = 0;
};

struct fg_pmft
{
    int kind;
    int naxes;
    PmftParams pp {};
    uint64_t nbins = 0;
    float jacobian = 1.0f;          // XY, XYT, XYZ: product of the bin widths
    std::vector<float> inv_jac;     // R12: 1 / (r_center * dr * dt1 * dt2) per r bin
    DevBuf hist;                    // uint64 per bin
    HostBox box {};
    uint32_t frames = 0, n_points = 0, n_query = 0;
    uint32_t n_equiv = 0xffffffffu; // XYZ: fixed by the first accumulate after a reset
};

struct fg_steinhardt
{
    std::vector<uint32_t> ls;
    bool average, wl, weighted, wl_normalize;
    uint32_t n = 0;
    StLs st {};
    size_t stride = 0; // sum of (2l + 1)
    DevBuf qlm, qlm_ave, ql, ql_ave, wlv, sys;
    DevBuf wl_terms; // Wigner-3j term classes of every l (launch_wl)
    WlTerms wt {};
    std::vector<std::vector<double>> w3j_host; // per l, for the system Wl (computed once)
    std::vector<float> order; // frames x n_l
    uint64_t bond_hint = 0;   // batched frames: bond slots the last one pass took (or the bonds counted)
    uint32_t frames = 1;
    bool computed = false;
};

namespace {

// Runs f, mapping exceptions to status codes.
template<typename F> fg_status guard(F&& f)
{
    try
    {
        f();
        return FG_OK;
    }
    catch (const Error& e)
    {
        g_last_error = e.what();
        return e.code;
    }
    catch (const std::bad_alloc&)
    {
        g_last_error = "host allocation failed";
        return FG_ERR_MEMORY;
    }
    catch (const std::exception& e)
    {
        g_last_error = e.what();
        return FG_ERR_RUNTIME;
    }
}

void require(const void* p, const char* what)
{
    if (p == nullptr)
    {
        value_error(std::string(what) + " must not be NULL");
    }
}

// Grid dims for a minimum cell width (nearest-plane distances / width, at least 1;
// 2D boxes are one cell deep). The grid is coarsened to at most ~2 cells per point.
void grid_dims(const HostBox& b, float width, uint32_t n, int dim[3])
{
    float pd[3];
    nearest_plane(b, pd);
    for (int a = 0; a < 3; ++a)
    {
        double d = std::floor(static_cast<double>(pd[a]) / static_cast<double>(width));
        if (!(d >= 1.0))
            d = 1.0;
        if (d > 2048.0)
            d = 2048.0;
        dim[a] = static_cast<int>(d);
    }
    if (b.is2d)
        dim[2] = 1;
    const double limit = 2.0 * n + 64.0;
    while (static_cast<double>(dim[0]) * dim[1] * dim[2] > limit)
    {
        for (int a = 0; a < (b.is2d ? 2 : 3); ++a)
            dim[a] = dim[a] > 1 ? (dim[a] * 3) / 4 : 1;
    }
}

// Builds (or reuses) the cell-sorted view of a point set for the given dims.
void build_grid(const DevBox& db, const float* dpts, uint32_t n, const int dim[3], GridEntry& g)
{
    cudaStream_t s = stream();
    g.dim[0] = dim[0];
    g.dim[1] = dim[1];
    g.dim[2] = dim[2];
    g.ncell = dim[0] * dim[1] * dim[2];
    DevBuf cell_of, rank, counts, scratch;
    cell_of.alloc(sizeof(uint32_t) * n);
    rank.alloc(sizeof(uint32_t) * n);
    counts.alloc(sizeof(uint32_t) * (g.ncell + 1));
    g.start.alloc(sizeof(uint32_t) * (g.ncell + 1));
    g.cpos.alloc(sizeof(float4) * n);
    g.cidx.alloc(sizeof(uint32_t) * n);
    scratch.alloc(scan_scratch_bytes(g.ncell + 1));
    FG_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(uint32_t) * (g.ncell + 1), s));
    launch_assign(db, dpts, n, dim, cell_of.as<uint32_t>(), rank.as<uint32_t>(), counts.as<uint32_t>(), s);
    scan_u32_to_u32(counts.as<uint32_t>(), g.start.as<uint32_t>(), g.ncell + 1, scratch.p, s);
    DevBuf cpos0, cidx0;
    cpos0.alloc(sizeof(float4) * n);
    cidx0.alloc(sizeof(uint32_t) * n);
    launch_scatter(db, dpts, n, cell_of.as<uint32_t>(), rank.as<uint32_t>(), g.start.as<uint32_t>(),
                   cpos0.as<float4>(), cidx0.as<uint32_t>(), s);
    // cells sorted by point index, so candidate sets are unions of sorted runs
    launch_sort_cells(g.start.as<uint32_t>(), g.ncell, cpos0.as<float4>(), cidx0.as<uint32_t>(), g.cpos.as<float4>(),
                      g.cidx.as<uint32_t>(), s);
    FG_CUDA(cudaGetLastError());
}

GridEntry& nq_grid(fg_nq* nq, const int dim[3])
{
    for (auto& g : nq->grids)
    {
        if (g->dim[0] == dim[0] && g->dim[1] == dim[1] && g->dim[2] == dim[2])
            return *g;
    }
    if (nq->grids.size() >= 4)
        nq->grids.erase(nq->grids.begin());
    nq->grids.push_back(std::make_unique<GridEntry>());
    build_grid(nq->dbox, nq->dpts, nq->n, dim, *nq->grids.back());
    return *nq->grids.back();
}

DevGrid view(const GridEntry& g)
{
    DevGrid d;
    d.dim[0] = g.dim[0];
    d.dim[1] = g.dim[1];
    d.dim[2] = g.dim[2];
    d.ncell = g.ncell;
    d.start = g.start.as<uint32_t>();
    d.cpos = g.cpos.as<float4>();
    d.cidx = g.cidx.as<uint32_t>();
    if (g.ghost)
    {
        d.ghost = 1;
        for (int a = 0; a < 3; ++a)
            d.gmin[a] = g.gp.gmin[a];
        d.ginv = g.gp.ginv;
    }
    return d;
}

// Mode inference and the mode's required arguments (NeighborQuery.h:195-228, 278-292).
void infer_mode(fg_query_args& a)
{
    if (a.mode == FG_MODE_NONE)
    {
        if (a.num_neighbors != 0xffffffffu)
            a.mode = FG_MODE_NEAREST;
        else if (a.r_max != -1.0f)
            a.mode = FG_MODE_BALL;
    }
    if (a.mode == FG_MODE_BALL)
    {
        if (a.r_max == -1.0f)
            runtime_error("You must set r_max in the query arguments when performing ball queries.");
        if (a.num_neighbors != 0xffffffffu)
            runtime_error("You cannot set num_neighbors in the query arguments when performing ball queries.");
    }
    else if (a.mode == FG_MODE_NEAREST)
    {
        if (a.num_neighbors == 0xffffffffu)
            runtime_error("You must set num_neighbors in the query arguments when performing number of neighbor "
                          "queries.");
        if (a.r_max == -1.0f)
            a.r_max = std::numeric_limits<float>::infinity();
    }
    else
    {
        runtime_error("Unknown mode");
    }
}

// QueryArgs validation: inference, then the per-point iterator checks
// (NeighborQuery.h:315-329).
void validate_args(fg_query_args& a)
{
    infer_mode(a);
    if (a.r_max <= 0.0f)
        value_error("NeighborQuery requires r_max to be positive.");
    if (a.r_max <= a.r_min)
        value_error("NeighborQuery requires that r_max must be greater than r_min.");
}

// CellQuery::validateQueryArgs (CellQuery.h:173-199): ball queries only, 2 r_max
// below every nearest-plane distance, then its own r_max checks.
void validate_cellquery_args(const HostBox& box, fg_query_args& a)
{
    infer_mode(a);
    if (a.mode == FG_MODE_NEAREST)
        runtime_error("CellQuery only supports ball queries (r_max), not nearest queries (num_neighbors). Use "
                      "AABBQuery for nearest neighbor queries.");
    float pd[3];
    nearest_plane(box, pd);
    if (pd[0] <= a.r_max * 2.0f || pd[1] <= a.r_max * 2.0f || (!box.is2d && pd[2] <= a.r_max * 2.0f))
        runtime_error("The CellQuery r_max is too large for this box.");
    if (a.r_max <= 0.0f)
        value_error("r_max must be positive.");
    if (a.r_max <= a.r_min)
        value_error("r_max must be greater than r_min.");
}

// CellQuery::setupGrid (CellQuery.h:143-167) in float, plus the ghost rule's
// fractional r_cut and lattice vectors (CellQuery.cc:92-98).
GhostParams ghost_setup(const HostBox& b, const DevBox& db, float r_cut)
{
    GhostParams gp;
    gp.b = db;
    gp.ginv = fdiv(1.0f, r_cut);
    const float wx = fadd(fadd(b.L[0], fmul(b.L[1], std::abs(b.xy))), fmul(b.L[2], std::abs(b.xz)));
    const float wy = fadd(b.L[1], fmul(b.L[2], std::abs(b.yz)));
    const float wz = b.L[2];
    gp.dim[0] = static_cast<int>(fmul(wx, gp.ginv)) + 3;
    gp.dim[1] = static_cast<int>(fmul(wy, gp.ginv)) + 3;
    gp.dim[2] = static_cast<int>(fmul(wz, gp.ginv)) + 3;
    const float bmx = fadd(fmul(b.L[1], std::min(0.0f, b.xy)), fmul(b.L[2], std::min(0.0f, b.xz)));
    const float bmy = fmul(b.L[2], std::min(0.0f, b.yz));
    // Box::makeAbsolute({0, 0, 0}) (Box.h:212-222)
    float ax = fadd(db.lo[0], fmul(0.0f, b.L[0]));
    float ay = fadd(db.lo[1], fmul(0.0f, b.L[1]));
    float az = fadd(db.lo[2], fmul(0.0f, b.L[2]));
    ax = fadd(ax, fadd(fmul(b.xy, ay), fmul(b.xz, az)));
    ay = fadd(ay, fmul(b.yz, az));
    if (b.is2d)
        az = 0.0f;
    gp.gmin[0] = fadd(fsub(bmx, r_cut), ax);
    gp.gmin[1] = fadd(fsub(bmy, r_cut), ay);
    gp.gmin[2] = fadd(-r_cut, az);
    float pd[3];
    nearest_plane(b, pd);
    for (int a = 0; a < 3; ++a)
        gp.fr[a] = fdiv(r_cut, pd[a]);
    const float lat[3][3] = {{b.L[0], 0.0f, 0.0f},
                             {fmul(b.L[1], b.xy), b.L[1], 0.0f},
                             {b.is2d ? 0.0f : fmul(b.L[2], b.xz), b.is2d ? 0.0f : fmul(b.L[2], b.yz),
                              b.is2d ? 0.0f : b.L[2]}};
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c)
            gp.lat[i][c] = lat[i][c];
    return gp;
}

// Counting sort of points (with_ghosts: and their ghosts) into the ghost grid.
void build_ghost_grid(const GhostParams& gp, const float* dpts, uint32_t n, int with_ghosts, GridEntry& g)
{
    cudaStream_t s = stream();
    g.ghost = true;
    g.gp = gp;
    g.dim[0] = gp.dim[0];
    g.dim[1] = gp.dim[1];
    g.dim[2] = gp.dim[2];
    const size_t ncell = static_cast<size_t>(gp.dim[0]) * gp.dim[1] * gp.dim[2];
    if (ncell >= (1ull << 31))
        runtime_error("The CellQuery grid is too large.");
    g.ncell = static_cast<int>(ncell);
    DevBuf copy_cell, copy_rank, counts, scratch, cpos0, cidx0;
    copy_cell.alloc(sizeof(uint32_t) * 8 * static_cast<size_t>(n));
    copy_rank.alloc(sizeof(uint32_t) * 8 * static_cast<size_t>(n));
    counts.alloc(sizeof(uint32_t) * (ncell + 2));
    g.start.alloc(sizeof(uint32_t) * (ncell + 2));
    scratch.alloc(scan_scratch_bytes(ncell + 2));
    FG_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(uint32_t) * (ncell + 2), s));
    launch_ghost_count(gp, dpts, n, with_ghosts, copy_cell.as<uint32_t>(), copy_rank.as<uint32_t>(),
                       counts.as<uint32_t>(), s);
    scan_u32_to_u32(counts.as<uint32_t>(), g.start.as<uint32_t>(), ncell + 2, scratch.p, s);
    uint32_t total = 0;
    FG_CUDA(cudaMemcpyAsync(&total, g.start.as<uint32_t>() + ncell + 1, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    sync();
    cpos0.alloc(sizeof(float4) * std::max<uint32_t>(total, 1));
    cidx0.alloc(sizeof(uint32_t) * std::max<uint32_t>(total, 1));
    g.cpos.alloc(sizeof(float4) * std::max<uint32_t>(total, 1));
    g.cidx.alloc(sizeof(uint32_t) * std::max<uint32_t>(total, 1));
    launch_ghost_scatter(gp, dpts, n, with_ghosts, copy_cell.as<uint32_t>(), copy_rank.as<uint32_t>(),
                         g.start.as<uint32_t>(), cpos0.as<float4>(), cidx0.as<uint32_t>(), s);
    // cells sorted by point index, so candidate sets are unions of sorted runs
    launch_sort_cells(g.start.as<uint32_t>(), g.ncell + 1, cpos0.as<float4>(), cidx0.as<uint32_t>(),
                      g.cpos.as<float4>(), g.cidx.as<uint32_t>(), s);
    FG_CUDA(cudaGetLastError());
}

void check_periodic(const HostBox& b)
{
    if (!(b.periodic[0] && b.periodic[1] && b.periodic[2]))
        throw Error(FG_ERR_VALUE, "Pair queries in a non-periodic box are not implemented.");
}

// A (box, points) system queries without the check above in the reference
// (RawPoints.h:50-62) and takes periodic images only along periodic axes
// (NeighborQuery.h:496-564). The cell grids here fold every axis, so a box that is
// not periodic on every axis is refused instead of answered with folded bonds.
void check_periodic_raw(const HostBox& b)
{
    if (!(b.periodic[0] && b.periodic[1] && b.periodic[2]))
        throw Error(FG_ERR_VALUE, "Pair queries of a (box, points) system in a box that is not periodic on every "
                                  "axis are not implemented.");
}

// The sorted query set: the object's own cell-sorted points, or the query points
// sorted into a grid with the same dims.
struct QuerySet
{
    const float4* qpos;
    const uint32_t* qidx;
    DevGrid qg;
    GridEntry own;
};

void make_query_set(fg_nq* nq, const GridEntry& g, const float* dq, uint32_t nqp, QuerySet& qs)
{
    if (dq == nullptr)
    {
        qs.qpos = g.cpos.as<float4>();
        qs.qidx = g.cidx.as<uint32_t>();
        qs.qg = view(g);
        return;
    }
    build_grid(nq->dbox, dq, nqp, g.dim, qs.own);
    qs.qpos = qs.own.cpos.as<float4>();
    qs.qidx = qs.own.cidx.as<uint32_t>();
    qs.qg = view(qs.own);
}

// Prefilter radii for the block-per-cell kernels (0 disables): wrap arithmetic only,
// >= 3 cells on every periodic axis, and r_max + delta below half the smallest
// nearest-plane distance, so the cell-derived image is the minimum image. delta
// bounds the difference between the cell-shifted float distance and the exact one.
//
// cull2 (count pass): candidates farther than sqrt(cull2) from the bounds of a
// cell's queries, in the same cell-shifted coordinates, are dropped before the
// merge. Valid for wrap arithmetic under the prefilter's conditions and for AABB
// arithmetic always (there each stencil entry is one image, and the cell-shifted
// vector approximates r = p_j - (q + image) within delta); not for ghost copies.
struct Prefilter
{
    float out2 = 0.0f;  // reject beyond
    float in2 = 0.0f;   // accept inside without the exact test (count pass, r_min == 0)
    float cull2 = 0.0f; // drop candidates beyond, per cell (count pass)
};

Prefilter prefilter(const fg_nq* nq, int arith, const int dim[3], float r_max, float r_min)
{
    Prefilter pf;
    if (arith != ARITH_WRAP && arith != ARITH_AABB)
        return pf;
    const double lmax = std::max(std::max(nq->box.L[0], nq->box.L[1]), nq->box.L[2]) *
        (1.0 + std::abs(nq->box.xy) + std::abs(nq->box.xz) + std::abs(nq->box.yz));
    // |prefilter distance - exact wrapped distance| is at most about 2.5e-6 lmax: each
    // coordinate of the cell-shifted difference carries a few roundings of magnitudes
    // up to lmax (2^-24 relative each), the exact box.wrap about 6.5 such roundings
    // plus the tilt terms'. Measured: at most 1.1e-5 on a 60^3 lattice (L = 60) and
    // on triclinic boxes of side 40. delta keeps twice the bound.
    const double delta = 5e-6 * (lmax + r_max) + 1e-6;
    const double ro = r_max + delta;
    if (arith == ARITH_AABB)
    {
        pf.cull2 = static_cast<float>(ro * ro * (1.0 + 1e-5));
        return pf;
    }
    if (dim[0] < 3 || dim[1] < 3 || (!nq->box.is2d && dim[2] < 3))
        return pf;
    float pd[3];
    nearest_plane(nq->box, pd);
    double minp = std::min(pd[0], pd[1]);
    if (!nq->box.is2d)
        minp = std::min(minp, static_cast<double>(pd[2]));
    if (!(r_max + delta < 0.5 * minp))
        return pf;
    pf.out2 = static_cast<float>(ro * ro * (1.0 + 1e-6));
    pf.cull2 = static_cast<float>(ro * ro * (1.0 + 1e-5));
    if (r_min == 0.0f && r_max > 2.0 * delta)
    {
        const double ri = r_max - delta;
        pf.in2 = static_cast<float>(ri * ri * (1.0 - 1e-6));
    }
    return pf;
}

// The CellQuery ghost grid for r_cut (cached on the NeighborQuery; the
// reference rebuilds it for every query, CellQuery.cc:26-30).
GridEntry& nq_ghost_grid(fg_nq* nq, float r_cut)
{
    for (auto& g : nq->ghost_grids)
    {
        if (g->r_cut == r_cut)
            return *g;
    }
    if (nq->ghost_grids.size() >= 2)
        nq->ghost_grids.erase(nq->ghost_grids.begin());
    nq->ghost_grids.push_back(std::make_unique<GridEntry>());
    GridEntry& g = *nq->ghost_grids.back();
    g.r_cut = r_cut;
    build_ghost_grid(ghost_setup(nq->box, nq->dbox, r_cut), nq->dpts, nq->n, 1, g);
    return g;
}

// Query points (the object's points when dq is NULL) in the cells of a ghost
// grid; points outside the grid go to the bucket past the last cell.
void make_ghost_query_set(fg_nq* nq, const GridEntry& g, const float* dq, uint32_t nqp, QuerySet& qs)
{
    build_ghost_grid(g.gp, dq != nullptr ? dq : nq->dpts, nqp, 0, qs.own);
    qs.qpos = qs.own.cpos.as<float4>();
    qs.qidx = qs.own.cidx.as<uint32_t>();
    qs.qg = view(qs.own);
}

// Count-pass kernel choice (fg_set_count_kernel): 0 automatic, 1 block-per-cell
// lanes over candidates only.
static int g_count_kernel = 0;

// Ball query -> NeighborList in reference order (count, scan, emit).
void ball_nlist(fg_nq* nq, const float* dq, uint32_t nqp, const fg_query_args& a, int by_distance, fg_nlist& out)
{
    cudaStream_t s = stream();
    const int arith =
        nq->kind == FG_NQ_LINKCELL ? ARITH_WRAP : (nq->kind == FG_NQ_CELLQUERY ? ARITH_GHOST : ARITH_AABB);
    if (arith == ARITH_AABB)
    {
        // updateImageVectors(r_max, true), NeighborQuery.h:504-509
        float pd[3];
        nearest_plane(nq->box, pd);
        if (pd[0] <= a.r_max * 2.0 || pd[1] <= a.r_max * 2.0 || (!nq->box.is2d && pd[2] <= a.r_max * 2.0))
            runtime_error("The AABBQuery r_max is too large for this box.");
    }
    int dim[3];
    QuerySet qs;
    GridEntry* gptr = nullptr;
    if (arith == ARITH_GHOST)
    {
        gptr = &nq_ghost_grid(nq, a.r_max);
        dim[0] = gptr->dim[0];
        dim[1] = gptr->dim[1];
        dim[2] = gptr->dim[2];
        make_ghost_query_set(nq, *gptr, dq, nqp, qs);
    }
    else
    {
        grid_dims(nq->box, a.r_max * (1.0f + 1e-5f), nq->n, dim);
        gptr = &nq_grid(nq, dim);
        make_query_set(nq, *gptr, dq, nqp, qs);
    }
    GridEntry& g = *gptr;
    BallParams p;
    p.r_max_sq = fmul(a.r_max, a.r_max);
    p.r_min_sq = fmul(a.r_min, a.r_min);
    p.exclude_ii = a.exclude_ii;
    p.arith = arith;
    p.nq = nqp;
    const Prefilter pf = prefilter(nq, arith, dim, a.r_max, a.r_min);
    DevBuf counts, offsets, scratch, heavy, heavy_n, over, over_n, gmask, gsorted, gtotal;
    counts.alloc(sizeof(uint32_t) * (nqp + 1));
    offsets.alloc(sizeof(uint64_t) * (nqp + 1));
    scratch.alloc(scan_scratch_bytes(nqp + 1));
    over.alloc(sizeof(uint32_t) * (nqp + 1));
    over_n.alloc(sizeof(uint32_t));
    const bool cellwise = !by_distance;
    // candidate capacity per cell: 4096 for dense point sets, whose 27-cell stencils
    // would overflow 1024 and fall back to the warp-per-query kernels
    const int cap = cell_cap_for(view(g), nq->n, nq->box.is2d && arith != ARITH_GHOST);
    if (cellwise)
    {
        gmask.alloc(sizeof(uint32_t) * static_cast<size_t>(nqp) * (cap / 32));
        gsorted.alloc(sizeof(uint32_t) * static_cast<size_t>(g.ncell) * cap);
        gtotal.alloc(sizeof(uint32_t) * static_cast<size_t>(std::max(g.ncell, 1)));
    }
    FG_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(uint32_t) * (nqp + 1), s));
    FG_CUDA(cudaMemsetAsync(over_n.p, 0, sizeof(uint32_t), s));
    reset_dev_err();
    uint32_t n_over = nqp;
    const uint32_t* list = nullptr;
    if (cellwise && g_count_kernel == 0 && arith == ARITH_WRAP && pf.out2 > 0.0f && pf.cull2 > 0.0f &&
        cap == CELL_CAP)
    {
        launch_nl_count(nq->dbox, view(g), qs.qg, p, pf.out2, pf.in2, pf.cull2, counts.as<uint32_t>(),
                        gmask.as<uint32_t>(), gsorted.as<uint32_t>(), gtotal.as<uint32_t>(), over.as<uint32_t>(),
                        over_n.as<uint32_t>(), s, nq->n);
        FG_CUDA(cudaMemcpyAsync(&n_over, over_n.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        sync();
        list = over.as<uint32_t>();
    }
    else if (cellwise)
    {
        // ghost grids hold copies of point indices; any index fits the same bound
        launch_cell_scan(0, nq->dbox, view(g), qs.qg, p, pf.out2, pf.in2, pf.cull2, counts.as<uint32_t>(),
                         gmask.as<uint32_t>(), gsorted.as<uint32_t>(), gtotal.as<uint32_t>(), over.as<uint32_t>(),
                         over_n.as<uint32_t>(), HistParams {}, nullptr, s, nq->n, cap);
        FG_CUDA(cudaMemcpyAsync(&n_over, over_n.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        sync();
        list = over.as<uint32_t>();
    }
    if (n_over > 0)
    {
        BallParams po = p;
        po.nq = n_over;
        launch_ball_count(nq->dbox, view(g), qs.qpos, qs.qidx, po, counts.as<uint32_t>(), s, list);
    }
    scan_u32_to_u64(counts.as<uint32_t>(), offsets.as<uint64_t>(), nqp + 1, scratch.p, s);
    uint64_t total = 0;
    FG_CUDA(cudaMemcpyAsync(&total, offsets.as<uint64_t>() + nqp, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    sync();
    if (total > 0xffffffffull)
        runtime_error("The query produced more than 2^32 - 1 bonds, beyond what a NeighborList can index.");
    out.nb = total;
    out.nq = nqp;
    out.np = nq->n;
    out.ij.alloc(sizeof(uint2) * total);
    out.dist.alloc(sizeof(float) * total);
    out.vec.alloc(sizeof(float) * 3 * total);
    out.unit_weights = true;
    out.seg_valid = false;
    heavy.alloc(sizeof(uint32_t) * (nqp + 1));
    heavy_n.alloc(sizeof(uint32_t));
    FG_CUDA(cudaMemsetAsync(heavy_n.p, 0, sizeof(uint32_t), s));
    if (cellwise)
    {
        launch_cell_emit(nq->dbox, view(g), qs.qg, p, gmask.as<uint32_t>(), gsorted.as<uint32_t>(),
                         gtotal.as<uint32_t>(), offsets.as<uint64_t>(), out.ij.as<uint2>(), out.dist.as<float>(),
                         out.vec.as<float>(), s, cap, counts.as<uint32_t>());
    }
    if (n_over > 0)
    {
        BallParams po = p;
        po.nq = n_over;
        launch_ball_emit(nq->dbox, view(g), qs.qpos, qs.qidx, po, counts.as<uint32_t>(), offsets.as<uint64_t>(),
                         by_distance, out.ij.as<uint2>(), out.dist.as<float>(), out.vec.as<float>(),
                         heavy.as<uint32_t>(), heavy_n.as<uint32_t>(), dev_err(), s, list);
        uint32_t nh = 0;
        FG_CUDA(cudaMemcpyAsync(&nh, heavy_n.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        sync();
        launch_ball_emit_heavy(nq->dbox, view(g), qs.qpos, qs.qidx, p, counts.as<uint32_t>(), offsets.as<uint64_t>(),
                               by_distance, heavy.as<uint32_t>(), nh, out.ij.as<uint2>(), out.dist.as<float>(),
                               out.vec.as<float>(), dev_err(), s);
    }
    FG_CUDA(cudaGetLastError());
    // segments / counts of the list straight from the query counts and offsets
    out.seg.alloc(sizeof(uint32_t) * std::max<uint32_t>(nqp, 1));
    launch_segments_from_offsets(counts.as<uint32_t>(), offsets.as<uint64_t>(), nqp, out.seg.as<uint32_t>(), s);
    out.cnt = std::move(counts);
    out.seg_valid = true;
    check_dev_err("ball query");
}

// kNN query -> NeighborList (AABBQuery.cc:152-281 / LinkCell.cc:575-679).
void knn_nlist(fg_nq* nq, const float* dq, uint32_t nqp, const fg_query_args& a, int by_distance, fg_nlist& out)
{
    cudaStream_t s = stream();
    const int arith = nq->kind == FG_NQ_LINKCELL ? ARITH_WRAP : ARITH_AABB;
    if (arith == ARITH_AABB)
    {
        // validateNearestNeighborArgs (NeighborQuery.h:235-270)
        if (a.scale != -1.0f && a.scale <= 1.0f)
            runtime_error("The scale query argument must be greater than 1.");
    }
    const uint32_t k = a.num_neighbors;
    if (k > knn_block_capacity() / 2)
        runtime_error("num_neighbors above " + std::to_string(knn_block_capacity() / 2) + " is not supported");
    // cell width ~1.5x the expected k-th neighbour distance (or r_max when smaller)
    const double vol = box_volume(nq->box);
    const double per = vol / std::max<uint32_t>(nq->n, 1) * std::max<uint32_t>(k, 1);
    double rk = nq->box.is2d ? std::sqrt(per / M_PI) : std::cbrt(3.0 * per / (4.0 * M_PI));
    // 1.3 x the mean k-th neighbour distance: queries whose k-th neighbour lies
    // beyond the stencil (rare: a ~4 sigma density fluctuation for k = 12) are
    // redone by the block brute force
    double width = 1.3 * rk;
    if (std::isfinite(a.r_max) && a.r_max * (1.0 + 1e-5) < width)
    {
        width = a.r_max * (1.0 + 1e-5);
    }
    int dim[3];
    grid_dims(nq->box, static_cast<float>(width), nq->n, dim);
    GridEntry& g = nq_grid(nq, dim);
    QuerySet qs;
    make_query_set(nq, g, dq, nqp, qs);
    float pd[3];
    nearest_plane(nq->box, pd);
    float covered = std::numeric_limits<float>::infinity();
    for (int ax = 0; ax < (nq->box.is2d ? 2 : 3); ++ax)
    {
        if (dim[ax] >= 3)
            covered = std::min(covered, static_cast<float>(static_cast<double>(pd[ax]) / dim[ax] * (1.0 - 1e-5)));
    }
    KnnParams p;
    p.r_max_sq = fmul(a.r_max, a.r_max);
    p.r_min = a.r_min;
    p.r_min_sq = fmul(a.r_min, a.r_min);
    p.exclude_ii = a.exclude_ii;
    p.arith = arith;
    p.k = k;
    p.nq = nqp;
    p.covered = covered;
    DevBuf tj, td, tv, counts, offsets, scratch, fail, fail_n;
    const size_t rows = static_cast<size_t>(nqp) * std::max<uint32_t>(k, 1);
    tj.alloc(sizeof(uint32_t) * rows);
    td.alloc(sizeof(float) * rows);
    tv.alloc(sizeof(float) * 3 * rows);
    counts.alloc(sizeof(uint32_t) * (nqp + 1));
    offsets.alloc(sizeof(uint64_t) * (nqp + 1));
    scratch.alloc(scan_scratch_bytes(nqp + 1));
    fail.alloc(sizeof(uint32_t) * (nqp + 1));
    fail_n.alloc(sizeof(uint32_t));
    FG_CUDA(cudaMemsetAsync(counts.p, 0, sizeof(uint32_t) * (nqp + 1), s));
    FG_CUDA(cudaMemsetAsync(fail_n.p, 0, sizeof(uint32_t), s));
    reset_dev_err();
    uint32_t nfail = 0;
    if (k == 0)
    {
        // nothing to find
    }
    else if (k <= 32)
    {
        launch_knn_warp(nq->dbox, view(g), qs.qpos, qs.qidx, p, tj.as<uint32_t>(), td.as<float>(), tv.as<float>(),
                        counts.as<uint32_t>(), fail.as<uint32_t>(), fail_n.as<uint32_t>(), s);
        FG_CUDA(cudaMemcpyAsync(&nfail, fail_n.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        sync();
    }
    else
    {
        std::vector<uint32_t> all(nqp);
        for (uint32_t t = 0; t < nqp; ++t)
            all[t] = t;
        FG_CUDA(cudaMemcpyAsync(fail.p, all.data(), sizeof(uint32_t) * nqp, cudaMemcpyHostToDevice, s));
        nfail = nqp;
    }
    if (nfail > 0)
    {
        launch_knn_block(nq->dbox, g.cpos.as<float4>(), g.cidx.as<uint32_t>(), nq->n, qs.qpos, qs.qidx, p,
                         fail.as<uint32_t>(), nfail, tj.as<uint32_t>(), td.as<float>(), tv.as<float>(),
                         counts.as<uint32_t>(), dev_err(), s);
    }
    FG_CUDA(cudaGetLastError());
    scan_u32_to_u64(counts.as<uint32_t>(), offsets.as<uint64_t>(), nqp + 1, scratch.p, s);
    uint64_t total = 0;
    FG_CUDA(cudaMemcpyAsync(&total, offsets.as<uint64_t>() + nqp, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    check_dev_err("nearest-neighbour query");
    out.nb = total;
    out.nq = nqp;
    out.np = nq->n;
    out.ij.alloc(sizeof(uint2) * total);
    out.dist.alloc(sizeof(float) * total);
    out.vec.alloc(sizeof(float) * 3 * total);
    out.unit_weights = true;
    launch_knn_compact(tj.as<uint32_t>(), td.as<float>(), tv.as<float>(), std::max<uint32_t>(k, 1), nqp,
                       counts.as<uint32_t>(), offsets.as<uint64_t>(), by_distance, out.ij.as<uint2>(),
                       out.dist.as<float>(), out.vec.as<float>(), s);
    out.seg.alloc(sizeof(uint32_t) * std::max<uint32_t>(nqp, 1));
    launch_segments_from_offsets(counts.as<uint32_t>(), offsets.as<uint64_t>(), nqp, out.seg.as<uint32_t>(), s);
    out.cnt = std::move(counts);
    out.seg_valid = true;
    FG_CUDA(cudaGetLastError());
    sync();
}

// The query arguments as a query of nq runs them (mode inferred), after the
// reference's checks of the box and the arguments.
fg_query_args checked_args(const fg_nq* nq, const fg_query_args* args)
{
    fg_query_args a = *args;
    if (nq->kind != FG_NQ_RAWPOINTS)
        check_periodic(nq->box);
    else
        check_periodic_raw(nq->box);
    if (nq->kind == FG_NQ_CELLQUERY)
        validate_cellquery_args(nq->box, a);
    else
        validate_args(a);
    return a;
}

void run_query(fg_nq* nq, const float* dq, uint32_t nqp, const fg_query_args* args, int by_distance, fg_nlist& out)
{
    const fg_query_args a = checked_args(nq, args);
    if (a.mode == FG_MODE_BALL)
        ball_nlist(nq, dq, nqp, a, by_distance, out);
    else
        knn_nlist(nq, dq, nqp, a, by_distance, out);
}

void ensure_segments(const fg_nlist* cnl)
{
    auto* nl = const_cast<fg_nlist*>(cnl);
    if (nl->seg_valid)
        return;
    nl->seg.alloc(sizeof(uint32_t) * std::max<uint32_t>(nl->nq, 1));
    nl->cnt.alloc(sizeof(uint32_t) * (std::max<uint32_t>(nl->nq, 1) + 1));
    launch_segments(nl->ij.as<uint2>(), nl->nb, nl->nq, nl->seg.as<uint32_t>(), nl->cnt.as<uint32_t>(), stream());
    FG_CUDA(cudaGetLastError());
    nl->seg_valid = true;
}

// Copies host points to a device buffer (N x 3 float32).
void upload_points(const float* host, uint32_t n, DevBuf& buf)
{
    buf.alloc(sizeof(float) * 3 * static_cast<size_t>(n));
    if (n > 0)
        FG_CUDA(cudaMemcpyAsync(buf.p, host, sizeof(float) * 3 * static_cast<size_t>(n), cudaMemcpyHostToDevice,
                                stream()));
}

// Second stream of the calling thread and device, for host-to-device copies that
// overlap kernels on the library stream, with the two events that order them.
struct CopyLane
{
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    int dev = -1;
};

CopyLane& copy_lane()
{
    static thread_local CopyLane c;
    int dev = 0;
    FG_CUDA(cudaGetDevice(&dev));
    if (c.s == nullptr || c.dev != dev)
    {
        FG_CUDA(cudaStreamCreateWithFlags(&c.s, cudaStreamNonBlocking));
        FG_CUDA(cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming));
        FG_CUDA(cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming));
        c.dev = dev;
    }
    return c;
}

// The object's own cell grid for a ball query with arguments a (the grid that
// ball_nlist looks up), built ahead of the query.
void prebuild_ball_grid(fg_nq* nq, const fg_query_args& a)
{
    if (a.mode != FG_MODE_BALL || nq->kind == FG_NQ_CELLQUERY)
        return;
    int dim[3];
    grid_dims(nq->box, a.r_max * (1.0f + 1e-5f), nq->n, dim);
    nq_grid(nq, dim);
}

// Copies n host query points to buf on the copy lane while the object's cell
// grid for the query is built on the library stream; the library stream waits
// for the copy before anything that follows. If the build fails, the copy is
// waited for before the error leaves (the caller may release its points then).
void upload_query_points(fg_nq* nq, const fg_query_args& a, const float* host, uint32_t n, DevBuf& buf)
{
    buf.alloc(sizeof(float) * 3 * static_cast<size_t>(n));
    if (n == 0)
        return;
    const cudaStream_t s = stream();
    CopyLane& c = copy_lane();
    FG_CUDA(cudaEventRecord(c.fork, s)); // the buffer's allocation is ordered on s
    FG_CUDA(cudaStreamWaitEvent(c.s, c.fork, 0));
    FG_CUDA(cudaMemcpyAsync(buf.p, host, sizeof(float) * 3 * static_cast<size_t>(n), cudaMemcpyHostToDevice, c.s));
    FG_CUDA(cudaEventRecord(c.join, c.s));
    try
    {
        prebuild_ball_grid(nq, a);
    }
    catch (...)
    {
        cudaStreamWaitEvent(s, c.join, 0);
        cudaStreamSynchronize(c.s);
        throw;
    }
    FG_CUDA(cudaStreamWaitEvent(s, c.join, 0));
}

// Whether n query points already on the device (dq) equal the object's points
// bit for bit; such a query runs on the object's own grid, as one with
// query_points == NULL does (equal words give identical pair arithmetic).
bool same_as_points(const fg_nq* nq, const float* dq, uint32_t n)
{
    if (n != nq->n || n == 0 || dq == nullptr)
        return false;
    if (dq == nq->dpts)
        return true;
    DevBuf flag;
    flag.alloc(sizeof(uint32_t));
    FG_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(uint32_t), stream()));
    launch_words_differ(reinterpret_cast<const uint32_t*>(dq), reinterpret_cast<const uint32_t*>(nq->dpts),
                        3ull * n, flag.as<uint32_t>(), stream());
    uint32_t differ = 1;
    FG_CUDA(cudaMemcpyAsync(&differ, flag.p, sizeof(differ), cudaMemcpyDeviceToHost, stream()));
    sync();
    return differ == 0;
}

void nq_init(fg_nq* nq, const fg_box* box, uint32_t n, int kind, float cell_width, const float* host_pts_for_check)
{
    if (kind < FG_NQ_RAWPOINTS || kind > FG_NQ_CELLQUERY)
        value_error("unknown neighbour-query kind");
    if (n == 0)
        value_error("Cannot create a NeighborQuery with 0 particles.");
    nq->box = to_host_box(box);
    nq->dbox = make_devbox(nq->box);
    nq->kind = kind;
    nq->n = n;
    if (nq->box.is2d && host_pts_for_check != nullptr)
    {
        for (uint32_t i = 0; i < n; ++i)
        {
            if (std::abs(host_pts_for_check[3 * static_cast<size_t>(i) + 2]) > 1e-6)
                value_error("A point with z != 0 was provided in a 2D box.");
        }
    }
    nq->cell_width = cell_width;
    if (kind == FG_NQ_LINKCELL)
    {
        // LinkCell.cc:222-260
        if (cell_width == 0.0f)
        {
            const uint32_t desired = std::max<uint32_t>(n / 10u, 1u);
            nq->cell_width = std::cbrt(fdiv(box_volume(nq->box), static_cast<float>(desired)));
        }
        float pd[3];
        nearest_plane(nq->box, pd);
        const double w2 = nq->cell_width * 2.0;
        if (w2 > pd[0] || w2 > pd[1] || (!nq->box.is2d && w2 > pd[2]))
            runtime_error("Cannot generate a cell list where cell_width is larger than half the box.");
    }
}

// Wigner 3j symbol (l l l; m1 m2 m3) by the Racah formula (long double factorials).
double wigner3j(int l, int m1, int m2, int m3)
{
    if (m1 + m2 + m3 != 0)
        return 0.0;
    auto lf = [](int x) { return std::lgamma(static_cast<long double>(x) + 1.0L); };
    const long double tri = 0.5L * (lf(l) + lf(l) + lf(l) - lf(3 * l + 1));
    const long double pre = 0.5L * (lf(l + m1) + lf(l - m1) + lf(l + m2) + lf(l - m2) + lf(l + m3) + lf(l - m3));
    const int kmin = std::max(0, std::max(-m1, m2));
    const int kmax = std::min(l, std::min(l - m1, l + m2));
    long double sum = 0.0L;
    for (int kk = kmin; kk <= kmax; ++kk)
    {
        const long double lt = lf(kk) + lf(l - kk) + lf(l - m1 - kk) + lf(l + m2 - kk) + lf(m1 + kk) + lf(kk - m2);
        const long double term = std::exp(tri + pre - lt);
        sum += (kk % 2) ? -term : term;
    }
    const int ph = -m3;
    return static_cast<double>(((ph % 2) != 0 ? -1.0L : 1.0L) * sum);
}

// Coefficients in the reference's iteration order (Wigner3j.cc:40-54).
std::vector<double> wigner3j_table(int l)
{
    std::vector<double> v;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        for (int m2 = std::max(-l - m1, -l); m2 <= std::min(l - m1, l); ++m2)
            v.push_back(wigner3j(l, m1, m2, -m1 - m2));
    }
    return v;
}

double reduce_w3j_host(const double* q, int l, const std::vector<double>& w)
{
    auto idx = [l](int m) { return m < 0 ? l - m : m; };
    double res = 0.0;
    size_t c = 0;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        for (int m2 = std::max(-l - m1, -l); m2 <= std::min(l - m1, l); ++m2, ++c)
        {
            const int m3 = -m1 - m2;
            const double* a = q + 2 * idx(m1);
            const double* b = q + 2 * idx(m2);
            const double* cc = q + 2 * idx(m3);
            const double abr = a[0] * b[0] - a[1] * b[1];
            const double abi = a[0] * b[1] + a[1] * b[0];
            res += w[c] * (abr * cc[0] - abi * cc[1]);
        }
    }
    return res;
}

} // namespace

namespace fg {
bool steinhardt_ball_single(fg_steinhardt* st, fg_nq* nq, const fg_query_args* args);
bool rdf_ball_single(fg_rdf* rdf, fg_nq* nq, const float* dq, const fg_query_args* args);
}

extern "C" {

const char* fg_last_error(void)
{
    return g_last_error.c_str();
}

int fg_version(void)
{
    return 1;
}

fg_status fg_set_stream(void* cuda_stream)
{
    return guard([&] {
        g_user_stream = static_cast<cudaStream_t>(cuda_stream);
        g_user_stream_set = cuda_stream != nullptr;
    });
}

// ---- NeighborQuery ----------------------------------------------------------------
fg_status fg_nq_create(const fg_box* box, const float* points, uint32_t n, int kind, float cell_width, fg_nq** out)
{
    return guard([&] {
        require(box, "box");
        require(out, "out");
        if (n > 0)
            require(points, "points");
        auto nq = std::make_unique<fg_nq>();
        nq_init(nq.get(), box, n, kind, cell_width, points);
        upload_points(points, n, nq->own);
        nq->dpts = nq->own.as<float>();
        sync();
        *out = nq.release();
    });
}

fg_status fg_nq_create_device(const fg_box* box, const float* device_points, uint32_t n, int kind, float cell_width,
                              fg_nq** out)
{
    return guard([&] {
        require(box, "box");
        require(out, "out");
        if (n > 0)
            require(device_points, "device_points");
        auto nq = std::make_unique<fg_nq>();
        nq_init(nq.get(), box, n, kind, cell_width, nullptr);
        nq->dpts = device_points;
        *out = nq.release();
    });
}

fg_status fg_nq_destroy(fg_nq* nq)
{
    return guard([&] {
        delete nq;
        sync();
    });
}

fg_status fg_nq_cell_width(const fg_nq* nq, float* out)
{
    return guard([&] {
        require(nq, "nq");
        *out = nq->cell_width;
    });
}

fg_status fg_nq_num_points(const fg_nq* nq, uint32_t* out)
{
    return guard([&] {
        require(nq, "nq");
        *out = nq->n;
    });
}

fg_status fg_nq_get_points(const fg_nq* nq, float* out)
{
    return guard([&] {
        require(nq, "nq");
        require(out, "out");
        FG_CUDA(cudaMemcpyAsync(out, nq->dpts, sizeof(float) * 3 * static_cast<size_t>(nq->n), cudaMemcpyDeviceToHost,
                                stream()));
        sync();
    });
}

fg_status fg_nq_query(fg_nq* nq, const float* query_points, uint32_t n_query, const fg_query_args* args,
                      int sort_by_distance, fg_nlist** out)
{
    return guard([&] {
        require(nq, "nq");
        require(args, "args");
        require(out, "out");
        DevBuf dq;
        const float* qp = nullptr;
        uint32_t nqp = nq->n;
        if (query_points != nullptr)
        {
            upload_query_points(nq, checked_args(nq, args), query_points, n_query, dq);
            if (!same_as_points(nq, dq.as<float>(), n_query))
            {
                qp = dq.as<float>();
                nqp = n_query;
            }
        }
        auto nl = std::make_unique<fg_nlist>();
        run_query(nq, qp, nqp, args, sort_by_distance, *nl);
        sync();
        *out = nl.release();
    });
}

fg_status fg_nq_query_device(fg_nq* nq, const float* device_query_points, uint32_t n_query, const fg_query_args* args,
                             int sort_by_distance, fg_nlist** out)
{
    return guard([&] {
        require(nq, "nq");
        require(args, "args");
        require(out, "out");
        auto nl = std::make_unique<fg_nlist>();
        const float* qp = (device_query_points == nq->dpts && n_query == nq->n) ? nullptr : device_query_points;
        run_query(nq, qp, qp ? n_query : nq->n, args, sort_by_distance, *nl);
        sync();
        *out = nl.release();
    });
}

// ---- NeighborList -------------------------------------------------------------------
fg_status fg_nlist_from_arrays(uint64_t num_bonds, const uint32_t* qi, uint32_t num_query_points, const uint32_t* pi,
                               uint32_t num_points, const float* vectors, const float* weights, fg_nlist** out)
{
    return guard([&] {
        require(out, "out");
        if (num_bonds > 0)
        {
            require(qi, "query_point_indices");
            require(pi, "point_indices");
            require(vectors, "vectors");
        }
        // NeighborList.cc:62-80
        uint32_t last = 0;
        for (uint64_t b = 0; b < num_bonds; ++b)
        {
            if (qi[b] < last)
                value_error("NeighborList query_point_index must be sorted.");
            if (qi[b] >= num_query_points)
                value_error("NeighborList query_point_index values must be less than num_query_points.");
            if (pi[b] >= num_points)
                value_error("NeighborList point_index values must be less than num_points.");
            last = qi[b];
        }
        cudaStream_t s = stream();
        auto nl = std::make_unique<fg_nlist>();
        nl->nb = num_bonds;
        nl->nq = num_query_points;
        nl->np = num_points;
        DevBuf dqi, dpi;
        dqi.alloc(sizeof(uint32_t) * num_bonds);
        dpi.alloc(sizeof(uint32_t) * num_bonds);
        nl->ij.alloc(sizeof(uint2) * num_bonds);
        nl->dist.alloc(sizeof(float) * num_bonds);
        nl->vec.alloc(sizeof(float) * 3 * num_bonds);
        if (num_bonds > 0)
        {
            FG_CUDA(cudaMemcpyAsync(dqi.p, qi, sizeof(uint32_t) * num_bonds, cudaMemcpyHostToDevice, s));
            FG_CUDA(cudaMemcpyAsync(dpi.p, pi, sizeof(uint32_t) * num_bonds, cudaMemcpyHostToDevice, s));
            FG_CUDA(cudaMemcpyAsync(nl->vec.p, vectors, sizeof(float) * 3 * num_bonds, cudaMemcpyHostToDevice, s));
        }
        launch_from_arrays(dqi.as<uint32_t>(), dpi.as<uint32_t>(), nl->vec.as<float>(), num_bonds, nl->ij.as<uint2>(),
                           nl->dist.as<float>(), s);
        nl->unit_weights = true;
        if (weights != nullptr)
        {
            bool all_one = true;
            for (uint64_t b = 0; b < num_bonds; ++b)
            {
                if (weights[b] != 1.0f)
                {
                    all_one = false;
                    break;
                }
            }
            if (!all_one)
            {
                nl->unit_weights = false;
                nl->weights.alloc(sizeof(float) * num_bonds);
                FG_CUDA(cudaMemcpyAsync(nl->weights.p, weights, sizeof(float) * num_bonds, cudaMemcpyHostToDevice, s));
            }
        }
        FG_CUDA(cudaGetLastError());
        sync();
        *out = nl.release();
    });
}

fg_status fg_nlist_all_pairs(const fg_box* box, const float* points, uint32_t num_points, const float* query_points,
                             uint32_t num_query_points, int exclude_ii, fg_nlist** out)
{
    return guard([&] {
        require(box, "box");
        require(out, "out");
        const HostBox hb = to_host_box(box);
        const DevBox db = make_devbox(hb);
        const uint64_t nii = exclude_ii ? std::min(num_points, num_query_points) : 0u;
        const uint64_t nb = static_cast<uint64_t>(num_points) * num_query_points - nii;
        DevBuf dp, dq;
        upload_points(points, num_points, dp);
        upload_points(query_points, num_query_points, dq);
        auto nl = std::make_unique<fg_nlist>();
        nl->nb = nb;
        nl->nq = num_query_points;
        nl->np = num_points;
        nl->ij.alloc(sizeof(uint2) * nb);
        nl->dist.alloc(sizeof(float) * nb);
        nl->vec.alloc(sizeof(float) * 3 * nb);
        launch_all_pairs(db, dp.as<float>(), num_points, dq.as<float>(), num_query_points, exclude_ii, nb,
                         nl->ij.as<uint2>(), nl->dist.as<float>(), nl->vec.as<float>(), stream());
        FG_CUDA(cudaGetLastError());
        sync();
        *out = nl.release();
    });
}

fg_status fg_nlist_destroy(fg_nlist* nl)
{
    return guard([&] {
        delete nl;
        sync();
    });
}

fg_status fg_nlist_copy(const fg_nlist* src, fg_nlist** out)
{
    return guard([&] {
        require(src, "src");
        require(out, "out");
        cudaStream_t s = stream();
        auto nl = std::make_unique<fg_nlist>();
        nl->nb = src->nb;
        nl->nq = src->nq;
        nl->np = src->np;
        nl->unit_weights = src->unit_weights;
        nl->ij.alloc(sizeof(uint2) * src->nb);
        nl->dist.alloc(sizeof(float) * src->nb);
        nl->vec.alloc(sizeof(float) * 3 * src->nb);
        if (src->nb > 0)
        {
            FG_CUDA(cudaMemcpyAsync(nl->ij.p, src->ij.p, sizeof(uint2) * src->nb, cudaMemcpyDeviceToDevice, s));
            FG_CUDA(cudaMemcpyAsync(nl->dist.p, src->dist.p, sizeof(float) * src->nb, cudaMemcpyDeviceToDevice, s));
            FG_CUDA(cudaMemcpyAsync(nl->vec.p, src->vec.p, sizeof(float) * 3 * src->nb, cudaMemcpyDeviceToDevice, s));
            if (!src->unit_weights)
            {
                nl->weights.alloc(sizeof(float) * src->nb);
                FG_CUDA(cudaMemcpyAsync(nl->weights.p, src->weights.p, sizeof(float) * src->nb,
                                        cudaMemcpyDeviceToDevice, s));
            }
        }
        sync();
        *out = nl.release();
    });
}

fg_status fg_nlist_num_bonds(const fg_nlist* nl, uint64_t* out)
{
    return guard([&] {
        require(nl, "nlist");
        *out = nl->nb;
    });
}

fg_status fg_nlist_num_query_points(const fg_nlist* nl, uint32_t* out)
{
    return guard([&] {
        require(nl, "nlist");
        *out = nl->nq;
    });
}

fg_status fg_nlist_num_points(const fg_nlist* nl, uint32_t* out)
{
    return guard([&] {
        require(nl, "nlist");
        *out = nl->np;
    });
}

fg_status fg_host_alloc(size_t bytes, void** out)
{
    return guard([&] {
        require(out, "out");
        *out = nullptr;
        if (bytes == 0)
            return;
        FG_CUDA(cudaMallocHost(out, bytes));
    });
}

fg_status fg_host_free(void* p)
{
    return guard([&] {
        if (p != nullptr)
            FG_CUDA(cudaFreeHost(p));
    });
}

fg_status fg_nlist_get(const fg_nlist* nl, uint32_t* neighbors, float* distances, float* weights, float* vectors)
{
    return guard([&] {
        require(nl, "nlist");
        cudaStream_t s = stream();
        if (nl->nb == 0)
            return;
        if (neighbors != nullptr)
            FG_CUDA(cudaMemcpyAsync(neighbors, nl->ij.p, sizeof(uint2) * nl->nb, cudaMemcpyDeviceToHost, s));
        if (distances != nullptr)
            FG_CUDA(cudaMemcpyAsync(distances, nl->dist.p, sizeof(float) * nl->nb, cudaMemcpyDeviceToHost, s));
        if (vectors != nullptr)
            FG_CUDA(cudaMemcpyAsync(vectors, nl->vec.p, sizeof(float) * 3 * nl->nb, cudaMemcpyDeviceToHost, s));
        if (weights != nullptr)
        {
            if (nl->unit_weights)
            {
                std::fill(weights, weights + nl->nb, 1.0f);
            }
            else
            {
                FG_CUDA(cudaMemcpyAsync(weights, nl->weights.p, sizeof(float) * nl->nb, cudaMemcpyDeviceToHost, s));
            }
        }
        sync();
    });
}

fg_status fg_nlist_device_arrays(const fg_nlist* nl, const uint32_t** neighbors, const float** distances,
                                 const float** vectors)
{
    return guard([&] {
        require(nl, "nlist");
        if (neighbors)
            *neighbors = nl->ij.as<uint32_t>();
        if (distances)
            *distances = nl->dist.as<float>();
        if (vectors)
            *vectors = nl->vec.as<float>();
    });
}

fg_status fg_nlist_segments(const fg_nlist* nl, uint32_t* segments, uint32_t* counts)
{
    return guard([&] {
        require(nl, "nlist");
        ensure_segments(nl);
        cudaStream_t s = stream();
        if (nl->nq > 0)
        {
            if (segments)
                FG_CUDA(cudaMemcpyAsync(segments, nl->seg.p, sizeof(uint32_t) * nl->nq, cudaMemcpyDeviceToHost, s));
            if (counts)
                FG_CUDA(cudaMemcpyAsync(counts, nl->cnt.p, sizeof(uint32_t) * nl->nq, cudaMemcpyDeviceToHost, s));
        }
        sync();
    });
}

fg_status fg_nlist_find_first_index(const fg_nlist* nl, uint32_t i, uint32_t* out)
{
    return guard([&] {
        require(nl, "nlist");
        if (nl->nb == 0)
        {
            *out = 0;
            return;
        }
        DevBuf r;
        r.alloc(sizeof(uint64_t));
        launch_first_index(nl->ij.as<uint2>(), nl->nb, i, r.as<uint64_t>(), stream());
        uint64_t h = 0;
        FG_CUDA(cudaMemcpyAsync(&h, r.p, sizeof(uint64_t), cudaMemcpyDeviceToHost, stream()));
        sync();
        *out = static_cast<uint32_t>(h);
    });
}

static void nlist_apply_keep(fg_nlist* nl, DevBuf& keep)
{
    cudaStream_t s = stream();
    DevBuf pos, scratch;
    pos.alloc(sizeof(uint64_t) * (nl->nb + 1));
    scratch.alloc(scan_scratch_bytes(nl->nb + 1));
    FG_CUDA(cudaMemsetAsync(keep.as<uint32_t>() + nl->nb, 0, sizeof(uint32_t), s));
    scan_u32_to_u64(keep.as<uint32_t>(), pos.as<uint64_t>(), nl->nb + 1, scratch.p, s);
    uint64_t total = 0;
    FG_CUDA(cudaMemcpyAsync(&total, pos.as<uint64_t>() + nl->nb, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
    sync();
    fg_nlist tmp;
    tmp.ij.alloc(sizeof(uint2) * total);
    tmp.dist.alloc(sizeof(float) * total);
    tmp.vec.alloc(sizeof(float) * 3 * total);
    if (!nl->unit_weights)
        tmp.weights.alloc(sizeof(float) * total);
    launch_compact(keep.as<uint32_t>(), pos.as<uint64_t>(), nl->nb, nl->ij.as<uint2>(), nl->dist.as<float>(),
                   nl->unit_weights ? nullptr : nl->weights.as<float>(), nl->vec.as<float>(), tmp.ij.as<uint2>(),
                   tmp.dist.as<float>(), nl->unit_weights ? nullptr : tmp.weights.as<float>(), tmp.vec.as<float>(), s);
    FG_CUDA(cudaGetLastError());
    nl->ij = std::move(tmp.ij);
    nl->dist = std::move(tmp.dist);
    nl->vec = std::move(tmp.vec);
    if (!nl->unit_weights)
        nl->weights = std::move(tmp.weights);
    nl->nb = total;
    nl->seg_valid = false;
    sync();
}

fg_status fg_nlist_filter(fg_nlist* nl, const uint8_t* keep_mask)
{
    return guard([&] {
        require(nl, "nlist");
        if (nl->nb == 0)
            return;
        require(keep_mask, "keep");
        DevBuf u8, keep;
        u8.alloc(nl->nb);
        keep.alloc(sizeof(uint32_t) * (nl->nb + 1));
        FG_CUDA(cudaMemcpyAsync(u8.p, keep_mask, nl->nb, cudaMemcpyHostToDevice, stream()));
        launch_keep_u8(u8.as<uint8_t>(), nl->nb, keep.as<uint32_t>(), stream());
        nlist_apply_keep(nl, keep);
    });
}

fg_status fg_nlist_filter_r(fg_nlist* nl, float r_max, float r_min)
{
    return guard([&] {
        require(nl, "nlist");
        if (r_max <= 0.0f)
            value_error("NeighborList.filter_r requires r_max to be positive.");
        if (r_min < 0.0f)
            value_error("NeighborList.filter_r requires r_min to be non-negative.");
        if (r_max <= r_min)
            value_error("NeighborList.filter_r requires that r_max must be greater than r_min.");
        if (nl->nb == 0)
            return;
        DevBuf keep;
        keep.alloc(sizeof(uint32_t) * (nl->nb + 1));
        launch_keep_r(nl->dist.as<float>(), nl->nb, r_max, r_min, keep.as<uint32_t>(), stream());
        nlist_apply_keep(nl, keep);
    });
}

fg_status fg_nlist_sort(fg_nlist* nl, int by_distance)
{
    // NeighborList::sort (NeighborList.cc:371-399): a post-processing utility, done on
    // the host copy of the bonds.
    return guard([&] {
        require(nl, "nlist");
        const uint64_t nb = nl->nb;
        if (nb == 0)
            return;
        std::vector<uint32_t> ij(2 * nb);
        std::vector<float> d(nb), w(nb), v(3 * nb);
        FG_CUDA(cudaMemcpyAsync(ij.data(), nl->ij.p, sizeof(uint2) * nb, cudaMemcpyDeviceToHost, stream()));
        FG_CUDA(cudaMemcpyAsync(d.data(), nl->dist.p, sizeof(float) * nb, cudaMemcpyDeviceToHost, stream()));
        FG_CUDA(cudaMemcpyAsync(v.data(), nl->vec.p, sizeof(float) * 3 * nb, cudaMemcpyDeviceToHost, stream()));
        if (!nl->unit_weights)
            FG_CUDA(cudaMemcpyAsync(w.data(), nl->weights.p, sizeof(float) * nb, cudaMemcpyDeviceToHost, stream()));
        else
            std::fill(w.begin(), w.end(), 1.0f);
        sync();
        std::vector<uint64_t> idx(nb);
        for (uint64_t b = 0; b < nb; ++b)
            idx[b] = b;
        auto less_tuple = [&](uint64_t a, uint64_t b) {
            if (ij[2 * a] != ij[2 * b])
                return ij[2 * a] < ij[2 * b];
            if (ij[2 * a + 1] != ij[2 * b + 1])
                return ij[2 * a + 1] < ij[2 * b + 1];
            if (w[a] != w[b])
                return w[a] < w[b];
            return d[a] < d[b];
        };
        auto less_dist = [&](uint64_t a, uint64_t b) {
            if (ij[2 * a] != ij[2 * b])
                return ij[2 * a] < ij[2 * b];
            if (d[a] != d[b])
                return d[a] < d[b];
            if (ij[2 * a + 1] != ij[2 * b + 1])
                return ij[2 * a + 1] < ij[2 * b + 1];
            return w[a] < w[b];
        };
        if (by_distance)
            std::stable_sort(idx.begin(), idx.end(), less_dist);
        else
            std::stable_sort(idx.begin(), idx.end(), less_tuple);
        std::vector<uint32_t> ij2(2 * nb);
        std::vector<float> d2(nb), w2(nb), v2(3 * nb);
        for (uint64_t b = 0; b < nb; ++b)
        {
            const uint64_t s = idx[b];
            ij2[2 * b] = ij[2 * s];
            ij2[2 * b + 1] = ij[2 * s + 1];
            d2[b] = d[s];
            w2[b] = w[s];
            v2[3 * b] = v[3 * s];
            v2[3 * b + 1] = v[3 * s + 1];
            v2[3 * b + 2] = v[3 * s + 2];
        }
        FG_CUDA(cudaMemcpyAsync(nl->ij.p, ij2.data(), sizeof(uint2) * nb, cudaMemcpyHostToDevice, stream()));
        FG_CUDA(cudaMemcpyAsync(nl->dist.p, d2.data(), sizeof(float) * nb, cudaMemcpyHostToDevice, stream()));
        FG_CUDA(cudaMemcpyAsync(nl->vec.p, v2.data(), sizeof(float) * 3 * nb, cudaMemcpyHostToDevice, stream()));
        if (!nl->unit_weights)
            FG_CUDA(cudaMemcpyAsync(nl->weights.p, w2.data(), sizeof(float) * nb, cudaMemcpyHostToDevice, stream()));
        nl->seg_valid = false;
        sync();
    });
}

// ---- RDF ------------------------------------------------------------------------------
fg_status fg_rdf_create(uint32_t bins, float r_max, float r_min, fg_rdf** out)
{
    return guard([&] {
        require(out, "out");
        // RDF.cc:27-42
        if (bins == 0)
            value_error("RDF requires a nonzero number of bins.");
        if (r_max <= 0.0f)
            value_error("RDF requires r_max to be positive.");
        if (r_min < 0.0f)
            value_error("RDF requires r_min to be non-negative.");
        if (r_max <= r_min)
            value_error("RDF requires that r_max must be greater than r_min.");
        auto r = std::make_unique<fg_rdf>();
        r->bins = bins;
        r->r_max = r_max;
        r->r_min = r_min;
        r->hist.alloc(sizeof(unsigned long long) * bins);
        FG_CUDA(cudaMemsetAsync(r->hist.p, 0, sizeof(unsigned long long) * bins, stream()));
        sync();
        *out = r.release();
    });
}

fg_status fg_rdf_destroy(fg_rdf* rdf)
{
    return guard([&] {
        delete rdf;
        sync();
    });
}

fg_status fg_rdf_set_mode(fg_rdf* rdf, int finite_size)
{
    return guard([&] {
        require(rdf, "rdf");
        rdf->finite_size = finite_size != 0;
    });
}

fg_status fg_rdf_reset(fg_rdf* rdf)
{
    return guard([&] {
        require(rdf, "rdf");
        FG_CUDA(cudaMemsetAsync(rdf->hist.p, 0, sizeof(unsigned long long) * rdf->bins, stream()));
        rdf->frames = 0;
        sync();
    });
}

static HistParams hist_params(const fg_rdf* r)
{
    HistParams h;
    h.h_min = r->r_min;
    h.h_max = r->r_max;
    // Histogram.h:130-131
    const float bw = fdiv(fsub(r->r_max, r->r_min), static_cast<float>(r->bins));
    h.h_inv = fdiv(1.0f, bw);
    h.bins = r->bins;
    return h;
}

// Single-frame (box, points) RDFs through the frames kernels (1) or the
// block-per-cell kernel of the NeighborQuery's own grid (0).
static bool g_rdf_single_frames = true;

static void rdf_accumulate(fg_rdf* rdf, fg_nq* nq, const float* dq, uint32_t nqp, const fg_nlist* nlist,
                           const fg_query_args* args)
{
    cudaStream_t s = stream();
    const HistParams h = hist_params(rdf);
    if (nlist != nullptr)
    {
        launch_hist_distances(nlist->dist.as<float>(), nlist->nb, h, rdf->hist.as<unsigned long long>(), s);
    }
    else if (g_rdf_single_frames && rdf_ball_single(rdf, nq, dq, args))
    {
        return; // frame counter, box and N updated by the frames path
    }
    else
    {
        require(args, "args");
        fg_query_args a = *args;
        if (nq->kind != FG_NQ_RAWPOINTS)
            check_periodic(nq->box);
        else
            check_periodic_raw(nq->box);
        if (nq->kind == FG_NQ_CELLQUERY)
            validate_cellquery_args(nq->box, a);
        else
            validate_args(a);
        if (a.mode == FG_MODE_BALL)
        {
            const int arith =
                nq->kind == FG_NQ_LINKCELL ? ARITH_WRAP : (nq->kind == FG_NQ_CELLQUERY ? ARITH_GHOST : ARITH_AABB);
            if (arith == ARITH_AABB)
            {
                float pd[3];
                nearest_plane(nq->box, pd);
                if (pd[0] <= a.r_max * 2.0 || pd[1] <= a.r_max * 2.0 || (!nq->box.is2d && pd[2] <= a.r_max * 2.0))
                    runtime_error("The AABBQuery r_max is too large for this box.");
            }
            int dim[3];
            QuerySet qs;
            GridEntry* gptr = nullptr;
            if (arith == ARITH_GHOST)
            {
                gptr = &nq_ghost_grid(nq, a.r_max);
                dim[0] = gptr->dim[0];
                dim[1] = gptr->dim[1];
                dim[2] = gptr->dim[2];
                make_ghost_query_set(nq, *gptr, dq, nqp, qs);
            }
            else
            {
                grid_dims(nq->box, a.r_max * (1.0f + 1e-5f), nq->n, dim);
                gptr = &nq_grid(nq, dim);
                make_query_set(nq, *gptr, dq, nqp, qs);
            }
            GridEntry& g = *gptr;
            BallParams p;
            p.r_max_sq = fmul(a.r_max, a.r_max);
            p.r_min_sq = fmul(a.r_min, a.r_min);
            p.exclude_ii = a.exclude_ii;
            p.arith = arith;
            p.nq = nqp;
            const Prefilter pf = prefilter(nq, p.arith, dim, a.r_max, a.r_min);
            // the histogram pass takes every cell (large stencils in tiles): no
            // queries are handed on, so it gets no overflow list
            launch_cell_scan(1, nq->dbox, view(g), qs.qg, p, pf.out2, 0.0f, 0.0f, nullptr, nullptr, nullptr, nullptr,
                             nullptr, nullptr, h, rdf->hist.as<unsigned long long>(), s);
            FG_CUDA(cudaGetLastError());
            sync();
        }
        else
        {
            fg_nlist tmp;
            knn_nlist(nq, dq, nqp, a, 0, tmp);
            launch_hist_distances(tmp.dist.as<float>(), tmp.nb, h, rdf->hist.as<unsigned long long>(), s);
            FG_CUDA(cudaGetLastError());
            sync();
        }
    }
    FG_CUDA(cudaGetLastError());
    // BondHistogramCompute::accumulateGeneral (BondHistogramCompute.h:115-126)
    rdf->box = nq->box;
    rdf->frames += 1;
    rdf->n_points = nq->n;
    rdf->n_query = nqp;
    sync();
}

fg_status fg_rdf_accumulate(fg_rdf* rdf, fg_nq* nq, const float* query_points, uint32_t n_query, const fg_nlist* nlist,
                            const fg_query_args* args)
{
    return guard([&] {
        require(rdf, "rdf");
        require(nq, "nq");
        DevBuf dq;
        const float* qp = nullptr;
        uint32_t nqp = nq->n;
        if (query_points != nullptr)
        {
            upload_points(query_points, n_query, dq);
            if (!same_as_points(nq, dq.as<float>(), n_query))
            {
                qp = dq.as<float>();
                nqp = n_query;
            }
        }
        rdf_accumulate(rdf, nq, qp, nqp, nlist, args);
    });
}

fg_status fg_rdf_accumulate_device(fg_rdf* rdf, fg_nq* nq, const float* device_query_points, uint32_t n_query,
                                   const fg_nlist* nlist, const fg_query_args* args)
{
    return guard([&] {
        require(rdf, "rdf");
        require(nq, "nq");
        const float* qp = (device_query_points == nq->dpts && n_query == nq->n) ? nullptr : device_query_points;
        rdf_accumulate(rdf, nq, qp, qp ? n_query : nq->n, nlist, args);
    });
}

static void rdf_edges(const fg_rdf* r, std::vector<float>& edges)
{
    // Histogram.h:126-138: edges[i] = min + float(i) * bin_width
    const float bw = fdiv(fsub(r->r_max, r->r_min), static_cast<float>(r->bins));
    edges.resize(r->bins + 1);
    for (uint32_t i = 0; i <= r->bins; ++i)
        edges[i] = fadd(r->r_min, fmul(static_cast<float>(i), bw));
}

fg_status fg_rdf_get(fg_rdf* rdf, uint32_t* bin_counts, float* rdf_out, float* n_r)
{
    return guard([&] {
        require(rdf, "rdf");
        std::vector<unsigned long long> h(rdf->bins);
        FG_CUDA(cudaMemcpyAsync(h.data(), rdf->hist.p, sizeof(unsigned long long) * rdf->bins, cudaMemcpyDeviceToHost,
                                stream()));
        sync();
        std::vector<uint32_t> c(rdf->bins);
        for (uint32_t i = 0; i < rdf->bins; ++i)
            c[i] = static_cast<uint32_t>(h[i]); // the reference's unsigned int bins
        if (bin_counts)
            std::memcpy(bin_counts, c.data(), sizeof(uint32_t) * rdf->bins);
        if (rdf_out == nullptr && n_r == nullptr)
            return;
        // RDF::reduce in float32 (RDF.cc:52-63, 73-99)
        std::vector<float> e;
        rdf_edges(rdf, e);
        const float volume_prefactor = static_cast<float>((4.0f / 3.0f) * M_PI);
        const float nqp = static_cast<float>(rdf->n_query);
        float number_density = fdiv(nqp, box_volume(rdf->box));
        if (rdf->finite_size)
            number_density = fmul(number_density, fdiv(static_cast<float>(rdf->n_query - 1), static_cast<float>(rdf->n_query)));
        const float np = static_cast<float>(rdf->n_points);
        const float nf = static_cast<float>(rdf->frames);
        const float prefactor = fdiv(1.0f, fmul(fmul(np, number_density), nf));
        for (uint32_t i = 0; i < rdf->bins; ++i)
        {
            const float r = e[i];
            const float nr = e[i + 1];
            float vol;
            if (rdf->box.is2d)
                vol = static_cast<float>(M_PI * static_cast<double>(fsub(fmul(nr, nr), fmul(r, r))));
            else
                vol = fmul(volume_prefactor, fsub(fmul(fmul(nr, nr), nr), fmul(fmul(r, r), r)));
            if (rdf_out)
                rdf_out[i] = fdiv(fmul(static_cast<float>(c[i]), prefactor), vol);
        }
        if (n_r)
        {
            const float pf2 = fdiv(1.0f, fmul(nqp, static_cast<float>(rdf->frames)));
            n_r[0] = fmul(static_cast<float>(c[0]), pf2);
            for (uint32_t i = 1; i < rdf->bins; ++i)
                n_r[i] = fadd(n_r[i - 1], fmul(static_cast<float>(c[i]), pf2));
        }
    });
}

fg_status fg_rdf_get_u64(fg_rdf* rdf, uint64_t* bin_counts, double* rdf_out, double* n_r)
{
    return guard([&] {
        require(rdf, "rdf");
        std::vector<unsigned long long> h(rdf->bins);
        FG_CUDA(cudaMemcpyAsync(h.data(), rdf->hist.p, sizeof(unsigned long long) * rdf->bins, cudaMemcpyDeviceToHost,
                                stream()));
        sync();
        if (bin_counts)
            for (uint32_t i = 0; i < rdf->bins; ++i)
                bin_counts[i] = h[i];
        // FP64 normalisation: shell volumes x density x frame count in double
        const double w = (static_cast<double>(rdf->r_max) - rdf->r_min) / rdf->bins;
        const double V = rdf->box.is2d ? static_cast<double>(rdf->box.L[0]) * rdf->box.L[1]
                                       : static_cast<double>(rdf->box.L[0]) * rdf->box.L[1] * rdf->box.L[2];
        double rho = rdf->n_query / V;
        if (rdf->finite_size)
            rho *= (rdf->n_query - 1.0) / rdf->n_query;
        const double pre = 1.0 / (static_cast<double>(rdf->n_points) * rho * rdf->frames);
        double acc = 0.0;
        for (uint32_t i = 0; i < rdf->bins; ++i)
        {
            const double r0 = rdf->r_min + i * w;
            const double r1 = rdf->r_min + (i + 1) * w;
            const double vol = rdf->box.is2d ? M_PI * (r1 * r1 - r0 * r0) : 4.0 / 3.0 * M_PI * (r1 * r1 * r1 - r0 * r0 * r0);
            if (rdf_out)
                rdf_out[i] = static_cast<double>(h[i]) * pre / vol;
            acc += static_cast<double>(h[i]) / (static_cast<double>(rdf->n_query) * rdf->frames);
            if (n_r)
                n_r[i] = acc;
        }
    });
}

fg_status fg_rdf_bin_edges(const fg_rdf* rdf, float* edges, float* centers)
{
    return guard([&] {
        require(rdf, "rdf");
        std::vector<float> e;
        rdf_edges(rdf, e);
        if (edges)
            std::memcpy(edges, e.data(), sizeof(float) * (rdf->bins + 1));
        if (centers)
            for (uint32_t i = 0; i < rdf->bins; ++i)
                centers[i] = fdiv(fadd(e[i], e[i + 1]), 2.0f);
    });
}

// ---- CorrelationFunction ------------------------------------------------------------
fg_status fg_cf_create(uint32_t bins, float r_max, fg_cf** out)
{
    return guard([&] {
        require(out, "out");
        // CorrelationFunction.cc:26-45
        if (bins == 0)
            value_error("CorrelationFunction  requires a nonzero number of bins.");
        if (r_max <= 0.0f)
            value_error("CorrelationFunction requires r_max to be positive.");
        auto c = std::make_unique<fg_cf>();
        c->bins = bins;
        c->r_max = r_max;
        c->sums.alloc(sizeof(double2) * bins);
        c->counts.alloc(sizeof(unsigned long long) * bins);
        FG_CUDA(cudaMemsetAsync(c->sums.p, 0, sizeof(double2) * bins, stream()));
        FG_CUDA(cudaMemsetAsync(c->counts.p, 0, sizeof(unsigned long long) * bins, stream()));
        sync();
        *out = c.release();
    });
}

fg_status fg_cf_destroy(fg_cf* cf)
{
    return guard([&] {
        delete cf;
        sync();
    });
}

fg_status fg_cf_reset(fg_cf* cf)
{
    return guard([&] {
        require(cf, "cf");
        FG_CUDA(cudaMemsetAsync(cf->sums.p, 0, sizeof(double2) * cf->bins, stream()));
        FG_CUDA(cudaMemsetAsync(cf->counts.p, 0, sizeof(unsigned long long) * cf->bins, stream()));
        cf->frames = 0;
        sync();
    });
}

static HistParams cf_hist_params(const fg_cf* c)
{
    // RegularAxis(bins, 0, r_max), Histogram.h:123-138
    HistParams h;
    h.h_min = 0.0f;
    h.h_max = c->r_max;
    const float bw = fdiv(c->r_max, static_cast<float>(c->bins));
    h.h_inv = fdiv(1.0f, bw);
    h.bins = c->bins;
    return h;
}

fg_status fg_cf_accumulate(fg_cf* cf, fg_nq* nq, const double* values, uint32_t n_values, const float* query_points,
                           uint32_t n_query, const double* query_values, uint32_t n_query_values,
                           const fg_nlist* nlist, const fg_query_args* args)
{
    return guard([&] {
        require(cf, "cf");
        require(nq, "nq");
        require(values, "values");
        if (n_values != nq->n)
            value_error("values must hold one value per point.");
        cudaStream_t s = stream();
        DevBuf dq;
        const float* qp = nullptr;
        uint32_t nqp = nq->n;
        if (query_points != nullptr)
        {
            upload_points(query_points, n_query, dq);
            if (!same_as_points(nq, dq.as<float>(), n_query))
            {
                qp = dq.as<float>();
                nqp = n_query;
            }
        }
        if (query_values == nullptr)
        {
            query_values = values;
            n_query_values = n_values;
        }
        if (n_query_values < nqp)
            value_error("query_values must hold one value per query point.");
        DevBuf dv, dqv;
        dv.alloc(sizeof(double2) * std::max<uint32_t>(n_values, 1));
        FG_CUDA(cudaMemcpyAsync(dv.p, values, sizeof(double2) * n_values, cudaMemcpyHostToDevice, s));
        const double2* qv = dv.as<double2>();
        if (query_values != values)
        {
            dqv.alloc(sizeof(double2) * std::max<uint32_t>(n_query_values, 1));
            FG_CUDA(cudaMemcpyAsync(dqv.p, query_values, sizeof(double2) * n_query_values, cudaMemcpyHostToDevice,
                                    s));
            qv = dqv.as<double2>();
        }
        fg_nlist tmp;
        const fg_nlist* bonds = nlist;
        if (nlist == nullptr)
        {
            require(args, "args");
            run_query(nq, qp, nqp, args, 0, tmp);
            bonds = &tmp;
        }
        else if (nlist->np > n_values || nlist->nq > n_query_values)
        {
            // the reference indexes values with the list's indices unchecked
            value_error("NeighborList found inconsistent array sizes.");
        }
        launch_cf_bonds(bonds->ij.as<uint2>(), bonds->dist.as<float>(), bonds->nb, dv.as<double2>(), qv,
                        cf_hist_params(cf), cf->sums.as<double2>(), cf->counts.as<unsigned long long>(), s);
        FG_CUDA(cudaGetLastError());
        // BondHistogramCompute::accumulateGeneral (BondHistogramCompute.h:115-126)
        cf->box = nq->box;
        cf->frames += 1;
        sync();
    });
}

fg_status fg_cf_get(fg_cf* cf, uint32_t* bin_counts, double* correlation)
{
    return guard([&] {
        require(cf, "cf");
        std::vector<unsigned long long> c(cf->bins);
        std::vector<double> sm(2 * static_cast<size_t>(cf->bins));
        FG_CUDA(cudaMemcpyAsync(c.data(), cf->counts.p, sizeof(unsigned long long) * cf->bins, cudaMemcpyDeviceToHost,
                                stream()));
        FG_CUDA(cudaMemcpyAsync(sm.data(), cf->sums.p, sizeof(double2) * cf->bins, cudaMemcpyDeviceToHost, stream()));
        sync();
        for (uint32_t i = 0; i < cf->bins; ++i)
        {
            // CorrelationFunction::reduce (CorrelationFunction.cc:48-59): sum / count
            // where the count is nonzero; the histogram holds unsigned int counts
            const uint32_t n = static_cast<uint32_t>(c[i]);
            if (bin_counts)
                bin_counts[i] = n;
            if (correlation)
            {
                double re = sm[2 * i], im = sm[2 * i + 1];
                if (n != 0)
                {
                    re /= static_cast<double>(n);
                    im /= static_cast<double>(n);
                }
                correlation[2 * i] = re;
                correlation[2 * i + 1] = im;
            }
        }
    });
}

fg_status fg_cf_bin_edges(const fg_cf* cf, float* edges, float* centers)
{
    return guard([&] {
        require(cf, "cf");
        // Histogram.h:126-138: edges[i] = min + float(i) * bin_width
        const float bw = fdiv(cf->r_max, static_cast<float>(cf->bins));
        std::vector<float> e(cf->bins + 1);
        for (uint32_t i = 0; i <= cf->bins; ++i)
            e[i] = fadd(0.0f, fmul(static_cast<float>(i), bw));
        if (edges)
            std::memcpy(edges, e.data(), sizeof(float) * (cf->bins + 1));
        if (centers)
            for (uint32_t i = 0; i < cf->bins; ++i)
                centers[i] = fdiv(fadd(e[i], e[i + 1]), 2.0f);
    });
}

fg_status fg_cf_state(const fg_cf* cf, fg_box* box, uint32_t* n_frames)
{
    return guard([&] {
        require(cf, "cf");
        if (box)
            *box = to_c_box(cf->box);
        if (n_frames)
            *n_frames = cf->frames;
    });
}

// ---- PMFT ------------------------------------------------------------------------------
namespace {
constexpr float PMFT_TWO_PI = 6.2831854820251465f; // float(2 pi) (Box.h:24)

PmftAxis pmft_axis(uint32_t n, float lo, float hi)
{
    // RegularAxis (Histogram.h:126-131)
    PmftAxis a;
    a.min = lo;
    a.max = hi;
    a.n = n;
    a.inv = fdiv(1.0f, fdiv(fsub(hi, lo), static_cast<float>(n)));
    return a;
}

float host_volume(const HostBox& b)
{
    // Box::getVolume (Box.h:196-205)
    return b.is2d ? fmul(b.L[0], b.L[1]) : fmul(fmul(b.L[0], b.L[1]), b.L[2]);
}
} // namespace

fg_status fg_pmft_create(int kind, const float* maxes, const uint32_t* bins, fg_pmft** out)
{
    return guard([&] {
        require(out, "out");
        require(maxes, "maxes");
        require(bins, "bins");
        auto pm = std::make_unique<fg_pmft>();
        pm->kind = kind;
        const char* name[4] = {"PMFTR12", "PMFTXYT", "PMFTXY", "PMFTXYZ"};
        if (kind < FG_PMFT_R12 || kind > FG_PMFT_XYZ)
            value_error("unknown PMFT kind");
        // constructors: PMFTR12.cc:28-80, PMFTXYT.cc:29-69, PMFTXY.cc:25-62, PMFTXYZ.cc:26-90
        const char* axis_names[4][3] = {{"R", "T1", "T2"}, {"X", "Y", "T"}, {"X", "Y", ""}, {"X", "Y", "Z"}};
        pm->naxes = kind == FG_PMFT_XY ? 2 : 3;
        for (int a = 0; a < pm->naxes; ++a)
            if (bins[a] < 1)
                value_error(std::string(name[kind]) + " requires at least 1 bin in " + axis_names[kind][a] + ".");
        if (kind == FG_PMFT_R12)
        {
            if (maxes[0] < 0.0f)
                value_error("PMFTR12 requires that r_max must be positive.");
            pm->pp.ax[0] = pmft_axis(bins[0], 0.0f, maxes[0]);
            pm->pp.ax[1] = pmft_axis(bins[1], 0.0f, PMFT_TWO_PI);
            pm->pp.ax[2] = pmft_axis(bins[2], 0.0f, PMFT_TWO_PI);
            const float dr = fdiv(maxes[0], static_cast<float>(bins[0]));
            const float dt1 = fdiv(PMFT_TWO_PI, static_cast<float>(bins[1]));
            const float dt2 = fdiv(1.0f, static_cast<float>(bins[2]));
            const float product = fmul(fmul(dr, dt1), dt2);
            const float bw = fdiv(maxes[0], static_cast<float>(bins[0]));
            pm->inv_jac.resize(bins[0]);
            for (uint32_t i = 0; i < bins[0]; ++i)
            {
                // bin centre (Histogram.h:87-95)
                const float e0 = fmul(static_cast<float>(i), bw);
                const float e1 = fmul(static_cast<float>(i + 1), bw);
                const float r = fdiv(fadd(e0, e1), 2.0f);
                pm->inv_jac[i] = fdiv(1.0f, fmul(r, product));
            }
        }
        else
        {
            const char* ax[3] = {"x_max", "y_max", "z_max"};
            const int nm = kind == FG_PMFT_XYZ ? 3 : 2;
            for (int a = 0; a < nm; ++a)
                if (maxes[a] < 0.0f)
                    value_error(std::string(name[kind]) + " requires that " + ax[a] + " must be positive.");
            float jac = 1.0f;
            for (int a = 0; a < nm; ++a)
            {
                pm->pp.ax[a] = pmft_axis(bins[a], -maxes[a], maxes[a]);
                const float d = fdiv(fmul(2.0f, maxes[a]), static_cast<float>(bins[a]));
                jac = a == 0 ? d : fmul(jac, d);
            }
            if (kind == FG_PMFT_XYT)
            {
                pm->pp.ax[2] = pmft_axis(bins[2], 0.0f, PMFT_TWO_PI);
                jac = fmul(jac, fdiv(1.0f, static_cast<float>(bins[2])));
            }
            pm->jacobian = jac;
        }
        if (pm->naxes == 2)
            pm->pp.ax[2] = pmft_axis(1, 0.0f, 1.0f);
        pm->nbins = static_cast<uint64_t>(pm->pp.ax[0].n) * pm->pp.ax[1].n * pm->pp.ax[2].n;
        pm->hist.alloc(sizeof(unsigned long long) * pm->nbins);
        FG_CUDA(cudaMemsetAsync(pm->hist.p, 0, sizeof(unsigned long long) * pm->nbins, stream()));
        sync();
        *out = pm.release();
    });
}

fg_status fg_pmft_destroy(fg_pmft* pm)
{
    return guard([&] {
        delete pm;
        sync();
    });
}

fg_status fg_pmft_reset(fg_pmft* pm)
{
    return guard([&] {
        require(pm, "pmft");
        FG_CUDA(cudaMemsetAsync(pm->hist.p, 0, sizeof(unsigned long long) * pm->nbins, stream()));
        pm->frames = 0;
        pm->n_equiv = 0xffffffffu;
        sync();
    });
}

fg_status fg_pmft_accumulate(fg_pmft* pm, fg_nq* nq, const float* orientations, uint32_t n_orient,
                             const float* query_points, uint32_t n_query, const float* query_orientations,
                             uint32_t n_query_orient, const float* equiv_orientations, uint32_t n_equiv,
                             const fg_nlist* nlist, const fg_query_args* args)
{
    return guard([&] {
        require(pm, "pmft");
        require(nq, "nq");
        cudaStream_t s = stream();
        // Box::enforce2D / enforce3D (Box.h:571-585)
        if (pm->kind == FG_PMFT_XYZ && nq->box.is2d)
            value_error("A 2D box was provided to a class that only supports 3D systems.");
        if (pm->kind != FG_PMFT_XYZ && !nq->box.is2d)
            value_error("A 3D box was provided to a class that only supports 2D systems.");
        DevBuf dq;
        const float* qp = nullptr;
        uint32_t nqp = nq->n;
        if (query_points != nullptr)
        {
            upload_points(query_points, n_query, dq);
            if (!same_as_points(nq, dq.as<float>(), n_query))
            {
                qp = dq.as<float>();
                nqp = n_query;
            }
        }
        const bool point_angles = pm->kind == FG_PMFT_R12 || pm->kind == FG_PMFT_XYT;
        if (point_angles)
        {
            require(orientations, "orientations");
            if (n_orient != nq->n)
                value_error("orientations must hold one angle per point.");
            if (query_orientations == nullptr)
            {
                query_orientations = orientations;
                n_query_orient = n_orient;
            }
        }
        require(query_orientations, "query_orientations");
        if (n_query_orient < nqp)
            value_error("query_orientations must hold one orientation per query point.");
        if (pm->kind == FG_PMFT_XYZ)
        {
            require(equiv_orientations, "equiv_orientations");
            // PMFTXYZ.cc:100-111
            if (pm->n_equiv == 0xffffffffu)
                pm->n_equiv = n_equiv;
            else if (pm->n_equiv != n_equiv)
                runtime_error("The number of equivalent orientations must be constant while accumulating data into "
                              "PMFTXYZ.");
        }
        DevBuf d_pa, d_qa, d_cs, d_quat, d_eq;
        if (point_angles)
        {
            d_pa.alloc(sizeof(float) * std::max<uint32_t>(n_orient, 1));
            FG_CUDA(cudaMemcpyAsync(d_pa.p, orientations, sizeof(float) * n_orient, cudaMemcpyHostToDevice, s));
            d_qa.alloc(sizeof(float) * std::max<uint32_t>(n_query_orient, 1));
            FG_CUDA(cudaMemcpyAsync(d_qa.p, query_orientations, sizeof(float) * n_query_orient,
                                    cudaMemcpyHostToDevice, s));
        }
        std::vector<float> cs;
        if (pm->kind == FG_PMFT_XYT || pm->kind == FG_PMFT_XY)
        {
            // rotmat2::fromAngle(-theta) (VectorMath.h:912-921): cos and sin from the C
            // library, once per query point
            cs.resize(2 * static_cast<size_t>(n_query_orient));
            for (uint32_t i = 0; i < n_query_orient; ++i)
            {
                const float th = -query_orientations[i];
                cs[2 * i] = std::cos(th);
                cs[2 * i + 1] = std::sin(th);
            }
            d_cs.alloc(sizeof(float2) * std::max<uint32_t>(n_query_orient, 1));
            FG_CUDA(cudaMemcpyAsync(d_cs.p, cs.data(), sizeof(float2) * n_query_orient, cudaMemcpyHostToDevice, s));
        }
        if (pm->kind == FG_PMFT_XYZ)
        {
            d_quat.alloc(sizeof(float4) * std::max<uint32_t>(n_query_orient, 1));
            FG_CUDA(cudaMemcpyAsync(d_quat.p, query_orientations, sizeof(float4) * n_query_orient,
                                    cudaMemcpyHostToDevice, s));
            d_eq.alloc(sizeof(float4) * std::max<uint32_t>(n_equiv, 1));
            if (n_equiv > 0)
                FG_CUDA(cudaMemcpyAsync(d_eq.p, equiv_orientations, sizeof(float4) * n_equiv, cudaMemcpyHostToDevice,
                                        s));
        }
        fg_nlist tmp;
        const fg_nlist* bonds = nlist;
        if (nlist == nullptr)
        {
            require(args, "args");
            run_query(nq, qp, nqp, args, 0, tmp);
            bonds = &tmp;
        }
        else if ((point_angles && nlist->np > n_orient) || nlist->nq > n_query_orient)
        {
            // the reference indexes the orientations with the list's indices unchecked
            value_error("NeighborList found inconsistent array sizes.");
        }
        PmftParams pp = pm->pp;
        pp.n_equiv = pm->kind == FG_PMFT_XYZ ? n_equiv : 0;
        launch_pmft_bonds(pm->kind, bonds->ij.as<uint2>(), bonds->dist.as<float>(), bonds->vec.as<float>(), bonds->nb,
                          d_pa.as<float>(), d_qa.as<float>(), d_cs.as<float2>(), d_quat.as<float4>(), d_eq.as<float4>(),
                          pp, pm->hist.as<unsigned long long>(), s);
        FG_CUDA(cudaGetLastError());
        // BondHistogramCompute::accumulateGeneral (BondHistogramCompute.h:115-126)
        pm->box = nq->box;
        pm->frames += 1;
        pm->n_points = nq->n;
        pm->n_query = nqp;
        sync();
    });
}

fg_status fg_pmft_get(fg_pmft* pm, uint32_t* bin_counts, float* pcf)
{
    return guard([&] {
        require(pm, "pmft");
        std::vector<unsigned long long> h(pm->nbins);
        FG_CUDA(cudaMemcpyAsync(h.data(), pm->hist.p, sizeof(unsigned long long) * pm->nbins, cudaMemcpyDeviceToHost,
                                stream()));
        sync();
        // PMFT::reduce (PMFT.h:70-82), PMFTXYZ::reduce (PMFTXYZ.cc:92-104): float32
        const float inv_num_dens = fdiv(host_volume(pm->box), static_cast<float>(pm->n_query));
        float denom = fmul(static_cast<float>(pm->frames), static_cast<float>(pm->n_points));
        if (pm->kind == FG_PMFT_XYZ)
            denom = fmul(denom, static_cast<float>(pm->n_equiv));
        const float norm_factor = fdiv(1.0f, denom);
        const float prefactor = fmul(inv_num_dens, norm_factor);
        const float jf = fdiv(1.0f, pm->jacobian);
        const uint64_t per_r = static_cast<uint64_t>(pm->pp.ax[1].n) * pm->pp.ax[2].n;
        for (uint64_t i = 0; i < pm->nbins; ++i)
        {
            const uint32_t c = static_cast<uint32_t>(h[i]);
            if (bin_counts)
                bin_counts[i] = c;
            if (pcf)
            {
                const float f = pm->kind == FG_PMFT_R12 ? pm->inv_jac[i / per_r] : jf;
                pcf[i] = fmul(fmul(static_cast<float>(c), prefactor), f);
            }
        }
    });
}

fg_status fg_pmft_axis(const fg_pmft* pm, int axis, float* edges, float* centers, float* bounds, uint32_t* n)
{
    return guard([&] {
        require(pm, "pmft");
        if (axis < 0 || axis >= pm->naxes)
            index_error("PMFT axis out of range");
        const PmftAxis& a = pm->pp.ax[axis];
        // RegularAxis edges / centres (Histogram.h:126-138, 87-95)
        const float bw = fdiv(fsub(a.max, a.min), static_cast<float>(a.n));
        std::vector<float> e(a.n + 1);
        for (uint32_t i = 0; i <= a.n; ++i)
            e[i] = fadd(a.min, fmul(static_cast<float>(i), bw));
        if (edges)
            std::memcpy(edges, e.data(), sizeof(float) * (a.n + 1));
        if (centers)
            for (uint32_t i = 0; i < a.n; ++i)
                centers[i] = fdiv(fadd(e[i], e[i + 1]), 2.0f);
        if (bounds)
        {
            bounds[0] = a.min;
            bounds[1] = a.max;
        }
        if (n)
            *n = a.n;
    });
}

fg_status fg_pmft_state(const fg_pmft* pm, fg_box* box, uint32_t* n_frames)
{
    return guard([&] {
        require(pm, "pmft");
        if (box)
            *box = to_c_box(pm->box);
        if (n_frames)
            *n_frames = pm->frames;
    });
}

fg_status fg_rdf_state(const fg_rdf* rdf, fg_box* box, uint32_t* n_frames, uint32_t* n_points, uint32_t* n_query)
{
    return guard([&] {
        require(rdf, "rdf");
        if (box)
            *box = to_c_box(rdf->box);
        if (n_frames)
            *n_frames = rdf->frames;
        if (n_points)
            *n_points = rdf->n_points;
        if (n_query)
            *n_query = rdf->n_query;
    });
}

fg_status fg_rdf_set_state(fg_rdf* rdf, const uint64_t* bin_counts, uint32_t n_frames, const fg_box* box,
                           uint32_t n_points, uint32_t n_query)
{
    return guard([&] {
        require(rdf, "rdf");
        require(bin_counts, "bin_counts");
        require(box, "box");
        FG_CUDA(cudaMemcpyAsync(rdf->hist.p, bin_counts, sizeof(unsigned long long) * rdf->bins,
                                cudaMemcpyHostToDevice, stream()));
        rdf->frames = n_frames;
        rdf->box = to_host_box(box);
        rdf->n_points = n_points;
        rdf->n_query = n_query;
        sync();
    });
}

// ---- Steinhardt ----------------------------------------------------------------------
fg_status fg_steinhardt_create(const uint32_t* ls, uint32_t n_l, int average, int wl, int weighted, int wl_normalize,
                               fg_steinhardt** out)
{
    return guard([&] {
        require(out, "out");
        if (n_l == 0)
            value_error("At least one l must be specified.");
        require(ls, "ls");
        if (n_l > static_cast<uint32_t>(ST_MAX_NL))
            value_error("at most " + std::to_string(ST_MAX_NL) + " values of l are supported per Steinhardt object");
        auto st = std::make_unique<fg_steinhardt>();
        st->ls.assign(ls, ls + n_l);
        st->average = average != 0;
        st->wl = wl != 0;
        st->weighted = weighted != 0;
        st->wl_normalize = wl_normalize != 0;
        st->st.nl = static_cast<int>(n_l);
        st->st.max_l = 0;
        for (uint32_t k = 0; k < n_l; ++k)
        {
            if (ls[k] > static_cast<uint32_t>(ST_MAX_L))
                value_error("l above " + std::to_string(ST_MAX_L) + " is not supported");
            st->st.l[k] = static_cast<int>(ls[k]);
            st->st.max_l = std::max(st->st.max_l, static_cast<int>(ls[k]));
            st->st.norm[k] = static_cast<float>(4.0 * M_PI / (2 * ls[k] + 1));
            st->stride += 2 * ls[k] + 1;
        }
        for (uint32_t k = 0; k < n_l; ++k)
            st->st.sorted_k[k] = static_cast<int>(k);
        std::stable_sort(st->st.sorted_k, st->st.sorted_k + n_l,
                         [&](int a, int b) { return st->st.l[a] < st->st.l[b]; });
        st_upload_tables(stream());
        std::vector<int4> terms;
        for (uint32_t k = 0; k < n_l; ++k)
        {
            st->w3j_host.emplace_back();
            if (st->wl)
            {
                st->w3j_host.back() = wigner3j_table(static_cast<int>(ls[k]));
                const std::vector<int4> t = wl_term_classes(static_cast<int>(ls[k]), wigner3j);
                st->wt.off[k] = static_cast<int>(terms.size());
                st->wt.cnt[k] = static_cast<int>(t.size());
                terms.insert(terms.end(), t.begin(), t.end());
            }
        }
        if (!terms.empty())
        {
            st->wl_terms.alloc(sizeof(int4) * terms.size());
            FG_CUDA(cudaMemcpyAsync(st->wl_terms.p, terms.data(), sizeof(int4) * terms.size(), cudaMemcpyHostToDevice,
                                    stream()));
        }
        sync();
        *out = st.release();
    });
}

fg_status fg_steinhardt_destroy(fg_steinhardt* st)
{
    return guard([&] {
        delete st;
        sync();
    });
}

// Steinhardt::normalizeSystem (Steinhardt.cc:291-327), in double, from the FP64
// system qlm sums of one frame (complex, every l's m in column order).
static void normalize_system(const fg_steinhardt* st, const double* sys, float* order)
{
    size_t col = 0;
    for (int k = 0; k < st->st.nl; ++k)
    {
        const int l = st->st.l[k];
        const double nf = 4.0 * M_PI / (2 * l + 1);
        double acc = 0.0;
        for (int m = 0; m < 2 * l + 1; ++m)
            acc += sys[2 * (col + m)] * sys[2 * (col + m)] + sys[2 * (col + m) + 1] * sys[2 * (col + m) + 1];
        const double qsys = std::sqrt(acc * nf);
        if (st->wl)
        {
            double v = reduce_w3j_host(&sys[2 * col], l, st->w3j_host[k]);
            if (st->wl_normalize)
            {
                const double w = std::sqrt(nf) / qsys;
                v *= w * w * w;
            }
            order[k] = static_cast<float>(v);
        }
        else
        {
            order[k] = static_cast<float>(qsys);
        }
        col += 2 * l + 1;
    }
}

fg_status fg_steinhardt_compute(fg_steinhardt* st, fg_nq* nq, const fg_nlist* nlist, const fg_query_args* args)
{
    return guard([&] {
        require(st, "steinhardt");
        require(nq, "nq");
        // the bond vectors are box.wrap(p_j - p_i), which here wraps every axis
        check_periodic_raw(nq->box);
        cudaStream_t s = stream();
        if (nlist == nullptr)
        {
            require(args, "args");
            if (steinhardt_ball_single(st, nq, args))
                return;
        }
        fg_nlist own;
        const fg_nlist* nl = nlist;
        if (nl == nullptr)
        {
            require(args, "args");
            run_query(nq, nullptr, nq->n, args, 0, own);
            nl = &own;
        }
        ensure_segments(nl);
        const uint32_t n = nq->n;
        st->n = n;
        st->frames = 1;
        // per-l offsets in one buffer
        size_t off = 0;
        for (int k = 0; k < st->st.nl; ++k)
        {
            st->st.qlm_offset[k] = off;
            off += static_cast<size_t>(n) * (2 * st->st.l[k] + 1);
        }
        st->qlm.alloc(sizeof(float2) * std::max<size_t>(off, 1));
        st->ql.alloc(sizeof(float) * std::max<size_t>(static_cast<size_t>(n) * st->st.nl, 1));
        const bool use_w = st->weighted && !nl->unit_weights;
        launch_qlm(nq->dbox, nq->dpts, n, nl->ij.as<uint2>(), nl->dist.as<float>(),
                   use_w ? nl->weights.as<float>() : nullptr, nl->seg.as<uint32_t>(), nl->cnt.as<uint32_t>(), st->st,
                   use_w ? 1 : 0, st->qlm.as<float2>(), st->ql.as<float>(), s, nullptr,
                   static_cast<double>(nl->nb) / std::max<uint32_t>(n, 1), st->wl ? 1 : 0);
        const float2* src = st->qlm.as<float2>();
        const float* qn = st->ql.as<float>();
        if (st->average)
        {
            st->qlm_ave.alloc(sizeof(float2) * std::max<size_t>(off, 1));
            st->ql_ave.alloc(sizeof(float) * std::max<size_t>(static_cast<size_t>(n) * st->st.nl, 1));
            launch_ave(n, nl->ij.as<uint2>(), nl->seg.as<uint32_t>(), nl->cnt.as<uint32_t>(), st->st, st->qlm.as<float2>(),
                       st->qlm_ave.as<float2>(), st->ql_ave.as<float>(), s);
            src = st->qlm_ave.as<float2>();
            qn = st->ql_ave.as<float>();
        }
        // system qlm: the frame-sum kernel over this single frame
        st->sys.alloc(sizeof(double) * 2 * st->stride);
        const uint32_t rows[2] = {0u, n};
        DevBuf d_rows, partial;
        d_rows.alloc(sizeof(rows));
        FG_CUDA(cudaMemcpyAsync(d_rows.p, rows, sizeof(rows), cudaMemcpyHostToDevice, s));
        partial.alloc(sizeof(double) * 2 * static_cast<size_t>(frames_sys_splits(n)) * st->stride);
        launch_frames_sys(d_rows.as<uint32_t>(), 1, n, st->st, static_cast<int>(st->stride), src, partial.as<double>(),
                          st->sys.as<double>(), s);
        if (st->wl)
        {
            st->wlv.alloc(sizeof(float) * std::max<size_t>(static_cast<size_t>(n) * st->st.nl, 1));
            launch_wl(n, st->st, st->wt, st->wl_terms.as<int4>(), src, qn, st->wl_normalize ? 1 : 0,
                      st->wlv.as<float>(), s);
        }
        FG_CUDA(cudaGetLastError());
        std::vector<double> sys(2 * st->stride);
        FG_CUDA(cudaMemcpyAsync(sys.data(), st->sys.p, sizeof(double) * 2 * st->stride, cudaMemcpyDeviceToHost, s));
        sync();
        st->order.assign(st->st.nl, 0.0f);
        normalize_system(st, sys.data(), st->order.data());
        st->computed = true;
    });
}

fg_status fg_steinhardt_num_particles(const fg_steinhardt* st, uint32_t* out)
{
    return guard([&] {
        require(st, "steinhardt");
        *out = st->n;
    });
}

fg_status fg_steinhardt_get(const fg_steinhardt* st, float* ql, float* particle_order, float* qlm, float* order)
{
    return guard([&] {
        require(st, "steinhardt");
        if (!st->computed)
            runtime_error("Steinhardt has not been computed");
        cudaStream_t s = stream();
        const size_t nl = static_cast<size_t>(st->n) * st->st.nl;
        const DevBuf& qlb = st->average ? st->ql_ave : st->ql;
        if (ql && nl)
            FG_CUDA(cudaMemcpyAsync(ql, qlb.p, sizeof(float) * nl, cudaMemcpyDeviceToHost, s));
        if (particle_order && nl)
        {
            const DevBuf& pb = st->wl ? st->wlv : qlb;
            FG_CUDA(cudaMemcpyAsync(particle_order, pb.p, sizeof(float) * nl, cudaMemcpyDeviceToHost, s));
        }
        if (qlm && st->n)
            FG_CUDA(cudaMemcpyAsync(qlm, st->qlm.p, sizeof(float2) * st->stride * st->n, cudaMemcpyDeviceToHost, s));
        if (order)
            std::memcpy(order, st->order.data(), sizeof(float) * st->order.size());
        sync();
    });
}


} // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free fused RDF histogram.
//
// For callers that cannot allocate device memory themselves or through this
// library: code running inside a framework that owns every device allocation
// (a simulation engine's analysis plugin handed device pointers, a custom
// allocator that forbids cudaMalloc/cudaMallocAsync mid-run, or work recorded
// into a CUDA graph by someone else). All scratch lives in one file-scope device
// array of fixed size, g_noalloc_scratch, held by every GPU that loads this
// library until the process exits. Host code never dereferences the array's
// name: its device address is obtained with cudaGetSymbolAddress, once per
// device, on the first call made with that device current (so that first call
// should come before any stream capture). Every call shares the array and it
// keeps the last call's contents; calls that overlap on the GPU race on it.
// ---------------------------------------------------------------------------
namespace {

constexpr uint32_t NOALLOC_MAX_POINTS = 1u << 16;                  // 65,536 points
constexpr uint32_t NOALLOC_MAX_CELLS = 2u * NOALLOC_MAX_POINTS + 64u; // grid_dims keeps <= 2N + 64 cells
constexpr size_t align256(size_t x) { return (x + 255) & ~static_cast<size_t>(255); }
constexpr size_t NA_CELL_OF = 0;
constexpr size_t NA_RANK = align256(NA_CELL_OF + 4ull * NOALLOC_MAX_POINTS);
constexpr size_t NA_COUNTS = align256(NA_RANK + 4ull * NOALLOC_MAX_POINTS);
constexpr size_t NA_START = align256(NA_COUNTS + 4ull * (NOALLOC_MAX_CELLS + 1));
constexpr size_t NA_CPOS0 = align256(NA_START + 4ull * (NOALLOC_MAX_CELLS + 1));
constexpr size_t NA_CIDX0 = align256(NA_CPOS0 + 16ull * NOALLOC_MAX_POINTS);
constexpr size_t NA_CPOS = align256(NA_CIDX0 + 4ull * NOALLOC_MAX_POINTS);
constexpr size_t NA_CIDX = align256(NA_CPOS + 16ull * NOALLOC_MAX_POINTS);
constexpr size_t NA_SCAN = align256(NA_CIDX + 4ull * NOALLOC_MAX_POINTS);
constexpr size_t NA_SCAN_BYTES = 8192; // scan_scratch_bytes(NOALLOC_MAX_CELLS + 1) is ~1.3 KB
constexpr size_t NOALLOC_SCRATCH_BYTES = align256(NA_SCAN + NA_SCAN_BYTES); // 4,203,520 bytes
static_assert(NOALLOC_SCRATCH_BYTES == 4203520, "the documented size of the allocation-free scratch");

__device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[64] = {nullptr};

// Device address of g_noalloc_scratch for the current device (looked up once per device).
unsigned char* noalloc_scratch()
{
    int dev = 0;
    FG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64)
        runtime_error("device ordinal out of range for the allocation-free entry point");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (g_noalloc_ptr[dev] == nullptr)
    {
        void* ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr)
            throw Error(FG_ERR_CUDA, std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(ptr);
    }
    return g_noalloc_ptr[dev];
}

} // namespace

extern "C" {

fg_status fg_rdf_histogram_noalloc(const fg_box* box, const float* device_points, uint32_t n, float r_max, float r_min,
                                   uint32_t bins, int exclude_ii, int kind, unsigned long long* device_counts,
                                   void* cuda_stream)
{
    return guard([&] {
        require(box, "box");
        require(device_points, "device_points");
        require(device_counts, "device_counts");
        if (n == 0)
            value_error("Cannot create a NeighborQuery with 0 particles.");
        if (n > NOALLOC_MAX_POINTS)
            value_error("fg_rdf_histogram_noalloc handles at most " + std::to_string(NOALLOC_MAX_POINTS) +
                        " points (its scratch is a fixed " + std::to_string(NOALLOC_SCRATCH_BYTES) +
                        "-byte device array); got " + std::to_string(n));
        if (bins == 0)
            value_error("RDF requires a nonzero number of bins.");
        if (r_max <= 0.0f)
            value_error("RDF requires r_max to be positive.");
        if (r_min < 0.0f)
            value_error("RDF requires r_min to be non-negative.");
        if (r_max <= r_min)
            value_error("RDF requires that r_max must be greater than r_min.");
        if (kind < FG_NQ_RAWPOINTS || kind > FG_NQ_LINKCELL)
            value_error("unknown neighbour-query kind");
        const HostBox hb = to_host_box(box);
        if (kind != FG_NQ_RAWPOINTS)
            check_periodic(hb);
        else
            check_periodic_raw(hb);
        const int arith = kind == FG_NQ_LINKCELL ? ARITH_WRAP : ARITH_AABB;
        float pd[3];
        nearest_plane(hb, pd);
        if (arith == ARITH_AABB &&
            (pd[0] <= r_max * 2.0 || pd[1] <= r_max * 2.0 || (!hb.is2d && pd[2] <= r_max * 2.0)))
            runtime_error("The AABBQuery r_max is too large for this box.");
        const DevBox db = make_devbox(hb);
        int dim[3];
        grid_dims(hb, r_max * (1.0f + 1e-5f), n, dim);
        const int ncell = dim[0] * dim[1] * dim[2];
        if (static_cast<uint32_t>(ncell) > NOALLOC_MAX_CELLS)
            runtime_error("cell grid larger than the allocation-free scratch");

        unsigned char* base = noalloc_scratch();
        cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
        uint32_t* cell_of = reinterpret_cast<uint32_t*>(base + NA_CELL_OF);
        uint32_t* rank = reinterpret_cast<uint32_t*>(base + NA_RANK);
        uint32_t* counts = reinterpret_cast<uint32_t*>(base + NA_COUNTS);
        uint32_t* start = reinterpret_cast<uint32_t*>(base + NA_START);
        float4* cpos0 = reinterpret_cast<float4*>(base + NA_CPOS0);
        uint32_t* cidx0 = reinterpret_cast<uint32_t*>(base + NA_CIDX0);
        float4* cpos = reinterpret_cast<float4*>(base + NA_CPOS);
        uint32_t* cidx = reinterpret_cast<uint32_t*>(base + NA_CIDX);
        void* scan_scratch = base + NA_SCAN;
        if (scan_scratch_bytes(static_cast<size_t>(ncell) + 1) > NA_SCAN_BYTES)
            runtime_error("scan scratch larger than reserved");

        // the cell counts start at zero; the output is this frame's counts
        FG_CUDA(cudaMemsetAsync(counts, 0, sizeof(uint32_t) * (ncell + 1), s));
        FG_CUDA(cudaMemsetAsync(device_counts, 0, sizeof(unsigned long long) * bins, s));
        launch_assign(db, device_points, n, dim, cell_of, rank, counts, s);
        scan_u32_to_u32(counts, start, static_cast<size_t>(ncell) + 1, scan_scratch, s);
        launch_scatter(db, device_points, n, cell_of, rank, start, cpos0, cidx0, s);
        launch_sort_cells(start, ncell, cpos0, cidx0, cpos, cidx, s);
        DevGrid g;
        g.dim[0] = dim[0];
        g.dim[1] = dim[1];
        g.dim[2] = dim[2];
        g.ncell = ncell;
        g.start = start;
        g.cpos = cpos;
        g.cidx = cidx;
        BallParams p;
        p.r_max_sq = fmul(r_max, r_max);
        p.r_min_sq = 0.0f;
        p.exclude_ii = exclude_ii != 0;
        p.arith = arith;
        p.nq = n;
        HistParams h;
        h.h_min = r_min;
        h.h_max = r_max;
        h.h_inv = fdiv(1.0f, fdiv(fsub(r_max, r_min), static_cast<float>(bins)));
        h.bins = bins;
        // a stub NeighborQuery carrying the box for the prefilter rule
        fg_nq probe;
        probe.box = hb;
        const Prefilter pf = prefilter(&probe, arith, dim, r_max, 0.0f);
        launch_cell_scan(1, db, g, g, p, pf.out2, 0.0f, 0.0f, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, h,
                         device_counts, s);
        FG_CUDA(cudaGetLastError());
    });
}

} // extern "C"

// ---------------------------------------------------------------------------
// Batched frames
//
// A batch is F frames of uneven N ((box, points) systems, AABB arithmetic as for
// RawPoints) held on the device once. RDF and Steinhardt over the batch run
// every frame in one launch per stage (fg_batch.cu) instead of one pipeline
// per frame, with the device-side sequence of each call recorded once as a
// CUDA graph and replayed while the batch layout and buffers stay the same.
// The histogram kernel's launch shape (stencil shell, warps per block, shared
// histogram copies) is chosen by timing the candidates on the first batch of
// each kind (density, r_max, bins) the process sees.
// ---------------------------------------------------------------------------

namespace {

bool g_graphs_enabled = true;
std::mutex g_tune_mu;
std::map<std::string, BatchHistConfig> g_tuned;
std::string g_tune_log;
BatchHistConfig g_forced {0, 0, 0};

struct GraphCache
{
    cudaGraphExec_t exec = nullptr;
    std::vector<uint64_t> key;
    uint64_t launches = 0;
    GraphCache() = default;
    GraphCache(const GraphCache&) = delete;
    GraphCache& operator=(const GraphCache&) = delete;
    ~GraphCache()
    {
        if (exec != nullptr)
            cudaGraphExecDestroy(exec);
    }
};

uint64_t fbits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, sizeof(u));
    return u;
}

// Runs body on the library stream, through a CUDA graph recorded on the first
// call with this key (body must only enqueue stream work on preallocated
// buffers). The legacy / per-thread default streams cannot be captured: there
// body runs directly.
template<typename F>
void run_graph(GraphCache& gc, bool allow, const std::vector<uint64_t>& key, const char* name, F&& body)
{
    cudaStream_t s = stream();
    const bool capturable =
        allow && g_graphs_enabled && s != nullptr && s != cudaStreamLegacy && s != cudaStreamPerThread;
    if (!capturable)
    {
        body();
        return;
    }
    if (gc.exec == nullptr || gc.key != key)
    {
        if (gc.exec != nullptr)
        {
            cudaGraphExecDestroy(gc.exec);
            gc.exec = nullptr;
        }
        FG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
        prof_begin_capture();
        try
        {
            body();
        }
        catch (...)
        {
            prof_end_capture();
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(s, &g);
            if (g != nullptr)
                cudaGraphDestroy(g);
            throw;
        }
        const uint64_t n = prof_end_capture();
        cudaGraph_t graph = nullptr;
        FG_CUDA(cudaStreamEndCapture(s, &graph));
        const cudaError_t e = cudaGraphInstantiate(&gc.exec, graph, 0);
        cudaGraphDestroy(graph);
        FG_CUDA(e);
        gc.key = key;
        gc.launches = n;
    }
    prof_add_launches(gc.launches);
    ProfScope prof_(name, s, false);
    FG_CUDA(cudaGraphLaunch(gc.exec, s));
}

// Cell grid of a batch for one cell width rule (r_max / shell), with its buffers.
struct BatchGridBufs
{
    uint64_t id = 0; // unique per grid built in this process (graph keys)
    float r_max = 0.0f;
    int shell = 0;
    uint32_t ncell = 0;
    std::vector<FrameDesc> fd_host;
    std::vector<uint32_t> cell_base_host;
    DevBuf fd, cell_base, counts, start, cell_of, rank, pos4, cpos0, cidx0, cpos, cidx, scan;
    DevBuf frame_out; // int per frame: some point outside the frame's box
};

} // namespace

struct fg_frames
{
    bool graphs = true; // record/replay CUDA graphs (off for one-off internal batches)
    std::vector<HostBox> boxes;
    std::vector<uint32_t> n;       // points per frame
    std::vector<uint32_t> pt_base; // nframes + 1
    uint32_t total = 0;
    DevBuf own;
    const float* dpts = nullptr;
    DevBuf d_pt_base;
    std::vector<std::unique_ptr<BatchGridBufs>> grids;
    // RDF workspace
    DevBuf queue;
    GraphCache rdf_graph;
    // Steinhardt workspace
    DevBuf st_counts, st_offsets, st_scan, st_j, st_vd, st_seg, st_partial, st_sys;
    GraphCache st_graph_a, st_graph_b, st_graph_one;
    DevBuf st_alloc; // one pass: bond slots taken
};

namespace {

// Grid of the batch for (r_max, shell): per-frame dims from the nearest-plane
// distances (at least `shell` cells on every periodic axis, else that frame
// falls back to shell 1 with r_max cells).
BatchGridBufs& batch_grid(fg_frames* fr, float r_max, int shell)
{
    for (auto& g : fr->grids)
    {
        if (g->r_max == r_max && g->shell == shell)
            return *g;
    }
    if (fr->grids.size() >= 4)
        fr->grids.erase(fr->grids.begin());
    static std::atomic<uint64_t> next_id {1};
    auto g = std::make_unique<BatchGridBufs>();
    g->id = next_id.fetch_add(1);
    g->r_max = r_max;
    g->shell = shell;
    const uint32_t F = static_cast<uint32_t>(fr->n.size());
    g->fd_host.resize(F);
    g->cell_base_host.resize(F + 1);
    uint64_t cells = 0;
    for (uint32_t f = 0; f < F; ++f)
    {
        const HostBox& hb = fr->boxes[f];
        int sh = shell;
        int dim[3];
        grid_dims(hb, fdiv(r_max, static_cast<float>(sh)) * (1.0f + 1e-5f), fr->n[f], dim);
        if (sh > 1 && (dim[0] < sh || dim[1] < sh || (!hb.is2d && dim[2] < sh)))
        {
            sh = 1;
            grid_dims(hb, r_max * (1.0f + 1e-5f), fr->n[f], dim);
        }
        FrameDesc& d = g->fd_host[f];
        d.b = make_devbox(hb);
        d.dim[0] = dim[0];
        d.dim[1] = dim[1];
        d.dim[2] = dim[2];
        d.shell = sh;
        d.cell_base = static_cast<uint32_t>(cells);
        d.ncell = static_cast<uint32_t>(dim[0] * dim[1] * dim[2]);
        d.pt_base = fr->pt_base[f];
        d.n = fr->n[f];
        g->cell_base_host[f] = static_cast<uint32_t>(cells);
        cells += d.ncell;
        if (cells >= (1ull << 31))
            runtime_error("the batch's cell grid exceeds 2^31 cells");
    }
    g->cell_base_host[F] = static_cast<uint32_t>(cells);
    g->ncell = static_cast<uint32_t>(cells);
    cudaStream_t s = stream();
    const uint32_t n = fr->total;
    g->fd.alloc(sizeof(FrameDesc) * F);
    g->frame_out.alloc(sizeof(int) * F);
    g->cell_base.alloc(sizeof(uint32_t) * (F + 1));
    g->counts.alloc(sizeof(uint32_t) * (g->ncell + 1));
    g->start.alloc(sizeof(uint32_t) * (g->ncell + 1));
    g->cell_of.alloc(sizeof(uint32_t) * n);
    g->rank.alloc(sizeof(uint32_t) * n);
    g->pos4.alloc(sizeof(float4) * n);
    g->cpos0.alloc(sizeof(float4) * n);
    g->cidx0.alloc(sizeof(uint32_t) * n);
    g->cpos.alloc(sizeof(float4) * n);
    g->cidx.alloc(sizeof(uint32_t) * n);
    g->scan.alloc(scan_scratch_bytes(static_cast<size_t>(g->ncell) + 1));
    FG_CUDA(cudaMemcpyAsync(g->fd.p, g->fd_host.data(), sizeof(FrameDesc) * F, cudaMemcpyHostToDevice, s));
    FG_CUDA(cudaMemcpyAsync(g->cell_base.p, g->cell_base_host.data(), sizeof(uint32_t) * (F + 1),
                            cudaMemcpyHostToDevice, s));
    sync(); // the host tables are pageable
    fr->grids.push_back(std::move(g));
    return *fr->grids.back();
}

// Enqueues the grid build (capturable: stream work on preallocated buffers only).
// sorted: each cell's points in index order (fixed bond order for Steinhardt's
// float sums); the histogram pass counts integers and needs no order.
void enqueue_grid_build(fg_frames* fr, BatchGridBufs& g, cudaStream_t s, bool sorted)
{
    const uint32_t F = static_cast<uint32_t>(fr->n.size());
    FG_CUDA(cudaMemsetAsync(g.counts.p, 0, sizeof(uint32_t) * (g.ncell + 1), s));
    FG_CUDA(cudaMemsetAsync(g.frame_out.p, 0, sizeof(int) * F, s));
    launch_frames_assign(g.fd.as<FrameDesc>(), fr->d_pt_base.as<uint32_t>(), F, fr->dpts, fr->total,
                         g.cell_of.as<uint32_t>(), g.rank.as<uint32_t>(), g.pos4.as<float4>(), g.counts.as<uint32_t>(),
                         g.frame_out.as<int>(), s);
    scan_u32_to_u32(g.counts.as<uint32_t>(), g.start.as<uint32_t>(), static_cast<size_t>(g.ncell) + 1, g.scan.p, s);
    if (!sorted)
    {
        launch_frames_scatter(fr->total, g.cell_of.as<uint32_t>(), g.rank.as<uint32_t>(), g.pos4.as<float4>(),
                              g.start.as<uint32_t>(), g.cpos.as<float4>(), g.cidx.as<uint32_t>(), s);
        return;
    }
    launch_frames_scatter(fr->total, g.cell_of.as<uint32_t>(), g.rank.as<uint32_t>(), g.pos4.as<float4>(),
                          g.start.as<uint32_t>(), g.cpos0.as<float4>(), g.cidx0.as<uint32_t>(), s);
    launch_sort_cells(g.start.as<uint32_t>(), static_cast<int>(g.ncell), g.cpos0.as<float4>(), g.cidx0.as<uint32_t>(),
                      g.cpos.as<float4>(), g.cidx.as<uint32_t>(), s);
}

BatchGrid batch_view(const fg_frames* fr, const BatchGridBufs& g)
{
    BatchGrid v;
    v.fd = g.fd.as<FrameDesc>();
    v.cell_base = g.cell_base.as<uint32_t>();
    v.nframes = static_cast<uint32_t>(fr->n.size());
    v.ncell = g.ncell;
    v.start = g.start.as<uint32_t>();
    v.cpos = g.cpos.as<float4>();
    v.cidx = g.cidx.as<uint32_t>();
    v.cell_of = g.cell_of.as<uint32_t>();
    v.frame_out = g.frame_out.as<int>();
    return v;
}

// Ball-query arguments of a batch call: checks shared with the per-frame path.
fg_query_args batch_args(const fg_frames* fr, const fg_query_args* args)
{
    fg_query_args a = *args;
    validate_args(a);
    if (a.mode != FG_MODE_BALL)
        value_error("batched frames support ball queries (r_max) only");
    for (const HostBox& hb : fr->boxes)
    {
        check_periodic(hb);
        float pd[3];
        nearest_plane(hb, pd);
        // updateImageVectors(r_max, true), NeighborQuery.h:504-509
        if (pd[0] <= a.r_max * 2.0 || pd[1] <= a.r_max * 2.0 || (!hb.is2d && pd[2] <= a.r_max * 2.0))
            runtime_error("The AABBQuery r_max is too large for this box.");
    }
    return a;
}

std::string tune_key(const fg_frames* fr, float r_max, uint32_t bins)
{
    double vol = 0.0;
    bool any2d = false;
    for (size_t f = 0; f < fr->boxes.size(); ++f)
    {
        const HostBox& b = fr->boxes[f];
        vol += b.is2d ? static_cast<double>(b.L[0]) * b.L[1] : static_cast<double>(b.L[0]) * b.L[1] * b.L[2];
        any2d = any2d || b.is2d;
    }
    const double per_cell = vol > 0.0 ? fr->total / vol * std::pow(static_cast<double>(r_max), any2d ? 2.0 : 3.0)
                                      : 0.0;
    const int dens = per_cell > 0.0 ? static_cast<int>(std::lround(2.0 * std::log2(per_cell))) : -99;
    // small frames behave differently (few cells to spread over the SMs): the
    // key also holds the size of the first frame, in powers of 4
    int size4 = 0;
    for (uint32_t n0 = fr->n.empty() ? 0u : fr->n[0]; n0 >= 4; n0 /= 4)
        ++size4;
    return std::string(any2d ? "2d" : "3d") + " pts_per_rmax_cell~2^" + std::to_string(dens / 2.0) +
           " first_frame~4^" + std::to_string(size4) + " bins_le_" +
           std::to_string(bins <= 1024 ? 1024 : (bins <= 2048 ? 2048 : 1 << 30));
}

// Chooses the histogram kernel's launch shape for this batch (cached per key):
// each candidate runs on the cells of the first frames (up to ~2^20 points) into
// a scratch histogram, best of three, timed with events on the stream.
BatchHistConfig tuned_config(fg_frames* fr, const BallParams& p, const HistParams& h, float r_max)
{
    if (g_forced.shell != 0)
        return g_forced;
    const std::string key = tune_key(fr, r_max, h.bins);
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end())
            return it->second;
    }
    cudaStream_t s = stream();
    // sample: the first frames, at least one, up to about 2^20 points
    const uint32_t F = static_cast<uint32_t>(fr->n.size());
    uint32_t nf = 1;
    while (nf < F && fr->pt_base[nf] < (1u << 20))
        ++nf;
    DevBuf scratch_hist;
    scratch_hist.alloc(sizeof(unsigned long long) * h.bins);
    if (fr->queue.bytes < sizeof(uint32_t))
        fr->queue.alloc(sizeof(uint32_t));
    cudaEvent_t e0, e1;
    FG_CUDA(cudaEventCreate(&e0));
    FG_CUDA(cudaEventCreate(&e1));
    BatchHistConfig best {1, 8, 1};
    float best_ms = std::numeric_limits<float>::infinity();
    std::string log = "rdf_frames [" + key + "]:";
    for (int shell = 1; shell <= 2; ++shell)
    {
        BatchGridBufs& g = batch_grid(fr, r_max, shell);
        enqueue_grid_build(fr, g, s, false);
        uint32_t limit = g.cell_base_host[nf];
        if (nf == 1 && fr->n[0] > (1u << 20))
        {
            // one large frame: a slab of its cells (cells run z-major, so the same
            // fraction of the box for either stencil)
            limit = static_cast<uint32_t>(static_cast<double>(limit) * (1u << 20) / fr->n[0]) + 1;
        }
        const BatchGrid v = batch_view(fr, g);
        for (int warps : {4, 8})
        {
            for (int copies : {1, 2, warps})
            {
                const BatchHistConfig cfg {shell, warps, copies};
                float ms = std::numeric_limits<float>::infinity();
                for (int rep = 0; rep < 3; ++rep)
                {
                    FG_CUDA(cudaMemsetAsync(fr->queue.p, 0, sizeof(uint32_t), s));
                    FG_CUDA(cudaMemsetAsync(scratch_hist.p, 0, sizeof(unsigned long long) * h.bins, s));
                    FG_CUDA(cudaEventRecord(e0, s));
                    launch_frames_hist(cfg, v, p, h, limit, fr->queue.as<uint32_t>(), scratch_hist.as<unsigned long long>(),
                                       s);
                    FG_CUDA(cudaEventRecord(e1, s));
                    FG_CUDA(cudaEventSynchronize(e1));
                    float t = 0.0f;
                    FG_CUDA(cudaEventElapsedTime(&t, e0, e1));
                    ms = std::min(ms, t);
                }
                char buf[96];
                std::snprintf(buf, sizeof(buf), " s%d/w%d/c%d=%.3fms", shell, warps, copies, ms);
                log += buf;
                if (ms < best_ms)
                {
                    best_ms = ms;
                    best = cfg;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    FG_CUDA(cudaGetLastError());
    char buf[96];
    std::snprintf(buf, sizeof(buf), " -> s%d/w%d/c%d\n", best.shell, best.warps, best.copies);
    log += buf;
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[key] = best;
    g_tune_log += log;
    return best;
}

void check_frames_points(const fg_box* boxes, const uint64_t* offsets, uint32_t n_frames)
{
    require(boxes, "boxes");
    require(offsets, "frame_offsets");
    if (n_frames == 0)
        value_error("a frame batch needs at least one frame");
    if (offsets[0] != 0)
        value_error("frame_offsets[0] must be 0");
    for (uint32_t f = 0; f < n_frames; ++f)
    {
        if (offsets[f + 1] <= offsets[f])
            value_error("Cannot create a NeighborQuery with 0 particles.");
    }
    if (offsets[n_frames] >= (1ull << 32))
        value_error("a frame batch holds fewer than 2^32 points");
}

fg_frames* new_frames(const fg_box* boxes, const uint64_t* offsets, uint32_t n_frames)
{
    check_frames_points(boxes, offsets, n_frames);
    auto fr = std::make_unique<fg_frames>();
    fr->boxes.resize(n_frames);
    fr->n.resize(n_frames);
    fr->pt_base.resize(n_frames + 1);
    for (uint32_t f = 0; f < n_frames; ++f)
    {
        fr->boxes[f] = to_host_box(&boxes[f]);
        fr->n[f] = static_cast<uint32_t>(offsets[f + 1] - offsets[f]);
        fr->pt_base[f] = static_cast<uint32_t>(offsets[f]);
    }
    fr->pt_base[n_frames] = static_cast<uint32_t>(offsets[n_frames]);
    fr->total = fr->pt_base[n_frames];
    fr->d_pt_base.alloc(sizeof(uint32_t) * (n_frames + 1));
    FG_CUDA(cudaMemcpyAsync(fr->d_pt_base.p, fr->pt_base.data(), sizeof(uint32_t) * (n_frames + 1),
                            cudaMemcpyHostToDevice, stream()));
    return fr.release();
}

} // namespace

extern "C" {

fg_status fg_frames_create(const fg_box* boxes, const float* points, const uint64_t* frame_offsets, uint32_t n_frames,
                           fg_frames** out)
{
    return guard([&] {
        require(out, "out");
        require(points, "points");
        std::unique_ptr<fg_frames> fr(new_frames(boxes, frame_offsets, n_frames));
        upload_points(points, fr->total, fr->own);
        fr->dpts = fr->own.as<float>();
        sync();
        *out = fr.release();
    });
}

fg_status fg_frames_create_list(const fg_box* boxes, const float* const* frame_points, const uint64_t* frame_offsets,
                                uint32_t n_frames, fg_frames** out)
{
    return guard([&] {
        require(out, "out");
        require(frame_points, "frame_points");
        std::unique_ptr<fg_frames> fr(new_frames(boxes, frame_offsets, n_frames));
        fr->own.alloc(sizeof(float) * 3 * std::max<size_t>(fr->total, 1));
        // one copy per frame straight into its slice: no host-side concatenation
        for (uint32_t f = 0; f < n_frames; ++f)
        {
            const uint64_t nf = frame_offsets[f + 1] - frame_offsets[f];
            if (nf == 0)
                continue;
            require(frame_points[f], "frame_points[f]");
            FG_CUDA(cudaMemcpyAsync(fr->own.as<float>() + 3 * frame_offsets[f], frame_points[f],
                                    sizeof(float) * 3 * nf, cudaMemcpyHostToDevice, stream()));
        }
        fr->dpts = fr->own.as<float>();
        sync();
        *out = fr.release();
    });
}

fg_status fg_frames_create_device(const fg_box* boxes, const float* device_points, const uint64_t* frame_offsets,
                                  uint32_t n_frames, fg_frames** out)
{
    return guard([&] {
        require(out, "out");
        require(device_points, "device_points");
        std::unique_ptr<fg_frames> fr(new_frames(boxes, frame_offsets, n_frames));
        fr->dpts = device_points;
        sync();
        *out = fr.release();
    });
}

fg_status fg_frames_set_points(fg_frames* fr, const float* points)
{
    return guard([&] {
        require(fr, "frames");
        require(points, "points");
        if (fr->own.p == nullptr)
            value_error("fg_frames_set_points needs a batch created from host points");
        FG_CUDA(cudaMemcpyAsync(fr->own.p, points, sizeof(float) * 3 * static_cast<size_t>(fr->total),
                                cudaMemcpyHostToDevice, stream()));
        sync();
    });
}

fg_status fg_frames_destroy(fg_frames* fr)
{
    return guard([&] {
        delete fr;
        sync();
    });
}

fg_status fg_frames_info(const fg_frames* fr, uint32_t* n_frames, uint64_t* n_points)
{
    return guard([&] {
        require(fr, "frames");
        if (n_frames)
            *n_frames = static_cast<uint32_t>(fr->n.size());
        if (n_points)
            *n_points = fr->total;
    });
}

static void rdf_frames(fg_rdf* rdf, fg_frames* fr, const fg_query_args& a)
{
    {
        cudaStream_t s = stream();
        BallParams p;
        p.r_max_sq = fmul(a.r_max, a.r_max);
        p.r_min_sq = fmul(a.r_min, a.r_min);
        p.exclude_ii = a.exclude_ii;
        p.arith = ARITH_AABB;
        p.nq = fr->total;
        const HistParams h = with_rsq_bins(hist_params(rdf), p.r_min_sq, p.r_max_sq);
        if (fr->queue.bytes < sizeof(uint32_t))
            fr->queue.alloc(sizeof(uint32_t));
        const BatchHistConfig cfg = tuned_config(fr, p, h, a.r_max);
        BatchGridBufs& g = batch_grid(fr, a.r_max, cfg.shell);
        const BatchGrid v = batch_view(fr, g);
        const std::vector<uint64_t> key = {reinterpret_cast<uint64_t>(rdf->hist.p), g.id,
                                           reinterpret_cast<uint64_t>(fr->dpts), static_cast<uint64_t>(cfg.shell),
                                           static_cast<uint64_t>(cfg.warps), static_cast<uint64_t>(cfg.copies),
                                           fbits(a.r_max), fbits(a.r_min), static_cast<uint64_t>(a.exclude_ii),
                                           static_cast<uint64_t>(h.bins), fbits(h.h_min), fbits(h.h_max)};
        run_graph(fr->rdf_graph, fr->graphs, key, "graph:rdf_frames", [&] {
            enqueue_grid_build(fr, g, s, false);
            FG_CUDA(cudaMemsetAsync(fr->queue.p, 0, sizeof(uint32_t), s));
            launch_frames_hist(cfg, v, p, h, g.ncell, fr->queue.as<uint32_t>(), rdf->hist.as<unsigned long long>(), s);
        });
        FG_CUDA(cudaGetLastError());
        sync();
        // F accumulate calls: the frame count grows by F, box and N are the last frame's
        rdf->frames += static_cast<uint32_t>(fr->n.size());
        rdf->box = fr->boxes.back();
        rdf->n_points = fr->n.back();
        rdf->n_query = fr->n.back();
    }
}

fg_status fg_rdf_accumulate_frames(fg_rdf* rdf, fg_frames* fr, const fg_query_args* args)
{
    return guard([&] {
        require(rdf, "rdf");
        require(fr, "frames");
        require(args, "args");
        const fg_query_args a = batch_args(fr, args);
        rdf_frames(rdf, fr, a);
    });
}

static void steinhardt_frames(fg_steinhardt* st, fg_frames* fr, const fg_query_args& a)
{
    cudaStream_t s = stream();
    const uint32_t P = fr->total;
    const uint32_t F = static_cast<uint32_t>(fr->n.size());
    BallParams p;
    p.r_max_sq = fmul(a.r_max, a.r_max);
    p.r_min_sq = fmul(a.r_min, a.r_min);
    p.exclude_ii = a.exclude_ii;
    p.arith = ARITH_AABB;
    p.nq = P;
    BatchGridBufs& g = batch_grid(fr, a.r_max, 1);
    const BatchGrid v = batch_view(fr, g);
    fr->st_counts.alloc(sizeof(uint32_t) * (P + 1));
    fr->st_seg.alloc(sizeof(uint32_t) * (P + 1));
    // outputs and per-frame sums
    st->n = P;
    st->frames = F;
    size_t off = 0;
    for (int k = 0; k < st->st.nl; ++k)
    {
        st->st.qlm_offset[k] = off;
        off += static_cast<size_t>(P) * (2 * st->st.l[k] + 1);
    }
    const int stride = static_cast<int>(st->stride);
    const uint32_t max_rows = *std::max_element(fr->n.begin(), fr->n.end());
    fr->st_partial.alloc(sizeof(double) * 2 * static_cast<size_t>(F) * frames_sys_splits(max_rows) * stride);
    fr->st_sys.alloc(sizeof(double) * 2 * static_cast<size_t>(F) * stride);
    st->qlm.alloc(sizeof(float2) * std::max<size_t>(off, 1));
    st->ql.alloc(sizeof(float) * std::max<size_t>(static_cast<size_t>(P) * st->st.nl, 1));
    if (st->average)
    {
        st->qlm_ave.alloc(sizeof(float2) * std::max<size_t>(off, 1));
        st->ql_ave.alloc(sizeof(float) * std::max<size_t>(static_cast<size_t>(P) * st->st.nl, 1));
    }
    if (st->wl)
        st->wlv.alloc(sizeof(float) * std::max<size_t>(static_cast<size_t>(P) * st->st.nl, 1));
    // expected bonds: N^2 / V times the ball volume per frame (uniform points)
    double expect = 0.0;
    for (uint32_t f = 0; f < F; ++f)
    {
        const HostBox& b = fr->boxes[f];
        const double r = a.r_max;
        const double vol = b.is2d ? static_cast<double>(b.L[0]) * b.L[1] : static_cast<double>(b.L[0]) * b.L[1] * b.L[2];
        const double ball = b.is2d ? M_PI * r * r : 4.0 / 3.0 * M_PI * r * r * r;
        expect += vol > 0.0 ? static_cast<double>(fr->n[f]) * fr->n[f] / vol * ball : 0.0;
    }
    // qlm, average, per-frame system sums, wl over the bonds (seg / counts / bond arrays)
    auto enqueue_rest = [&](double mean_bonds) {
        launch_qlm(g.fd_host[0].b, fr->dpts, P, nullptr, nullptr, nullptr, fr->st_seg.as<uint32_t>(),
                   fr->st_counts.as<uint32_t>(), st->st, 0, st->qlm.as<float2>(), st->ql.as<float>(), s,
                   fr->st_vd.as<float4>(), mean_bonds, st->wl ? 1 : 0);
        const float2* src = st->qlm.as<float2>();
        const float* qn = st->ql.as<float>();
        if (st->average)
        {
            launch_ave(P, nullptr, fr->st_seg.as<uint32_t>(), fr->st_counts.as<uint32_t>(), st->st, st->qlm.as<float2>(),
                       st->qlm_ave.as<float2>(), st->ql_ave.as<float>(), s, fr->st_j.as<uint32_t>(), v.cidx);
            src = st->qlm_ave.as<float2>();
            qn = st->ql_ave.as<float>();
        }
        launch_frames_sys(fr->d_pt_base.as<uint32_t>(), F, max_rows, st->st, stride, src, fr->st_partial.as<double>(),
                          fr->st_sys.as<double>(), s);
        if (st->wl)
        {
            launch_wl(P, st->st, st->wt, st->wl_terms.as<int4>(), src, qn, st->wl_normalize ? 1 : 0, st->wlv.as<float>(),
                      s);
        }
    };
    auto outputs_key = [&](std::vector<uint64_t> key) {
        for (const void* ptr : {fr->st_j.p, fr->st_vd.p, fr->st_seg.p, fr->st_counts.p, fr->st_partial.p, fr->st_sys.p,
                                st->qlm.p, st->ql.p, st->qlm_ave.p, st->ql_ave.p, st->wlv.p, st->wl_terms.p,
                                static_cast<void*>(st)})
            key.push_back(reinterpret_cast<uint64_t>(ptr));
        for (uint64_t x : {fbits(a.r_max), fbits(a.r_min), static_cast<uint64_t>(a.exclude_ii),
                           static_cast<uint64_t>(st->average), static_cast<uint64_t>(st->wl),
                           static_cast<uint64_t>(st->wl_normalize)})
            key.push_back(x);
        for (int k = 0; k < st->st.nl; ++k)
            key.push_back(static_cast<uint64_t>(st->st.l[k]));
        return key;
    };
    std::vector<double> sys(2 * static_cast<size_t>(F) * stride);
    bool done = false;
    // one pass: bonds placed by per-warp chunks, no counts beforehand; arrays sized by
    // the expected bonds or the last run's (whichever is larger) plus the chunk tails
    const uint64_t cap = static_cast<uint64_t>(std::max(1.25 * expect, 1.1 * static_cast<double>(st->bond_hint))) +
                         frames_ball_onepass_slack(g.ncell) + P;
    if (cap < (1ull << 32))
    {
        fr->st_j.alloc(sizeof(uint32_t) * cap);
        fr->st_vd.alloc(sizeof(float4) * cap);
        fr->st_alloc.alloc(sizeof(unsigned long long));
        std::vector<uint64_t> key = outputs_key({g.id, cap, reinterpret_cast<uint64_t>(fr->dpts),
                                                 reinterpret_cast<uint64_t>(fr->st_alloc.p)});
        run_graph(fr->st_graph_one, fr->graphs, key, "graph:steinhardt_frames", [&] {
            enqueue_grid_build(fr, g, s, true);
            FG_CUDA(cudaMemsetAsync(fr->st_alloc.p, 0, sizeof(unsigned long long), s));
            launch_frames_ball_onepass(v, p, P, fr->st_counts.as<uint32_t>(), fr->st_seg.as<uint32_t>(),
                                       fr->st_j.as<uint32_t>(), fr->st_vd.as<float4>(),
                                       fr->st_alloc.as<unsigned long long>(), cap, s);
            enqueue_rest(expect / std::max<uint32_t>(P, 1));
        });
        FG_CUDA(cudaGetLastError());
        unsigned long long taken = 0;
        FG_CUDA(cudaMemcpyAsync(&taken, fr->st_alloc.p, sizeof(taken), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaMemcpyAsync(sys.data(), fr->st_sys.p, sizeof(double) * sys.size(), cudaMemcpyDeviceToHost, s));
        sync();
        st->bond_hint = taken;
        done = taken <= cap;
    }
    if (!done)
    {
        // two passes: bond counts and offsets, then the bonds at their offsets
        fr->st_offsets.alloc(sizeof(uint64_t) * (P + 1));
        fr->st_scan.alloc(scan_scratch_bytes(static_cast<size_t>(P) + 1));
        const std::vector<uint64_t> key_a = {g.id, reinterpret_cast<uint64_t>(fr->dpts),
                                             reinterpret_cast<uint64_t>(fr->st_counts.p),
                                             reinterpret_cast<uint64_t>(fr->st_offsets.p),
                                             reinterpret_cast<uint64_t>(fr->st_scan.p), fbits(a.r_max), fbits(a.r_min),
                                             static_cast<uint64_t>(a.exclude_ii)};
        run_graph(fr->st_graph_a, fr->graphs, key_a, "graph:steinhardt_frames_count", [&] {
            enqueue_grid_build(fr, g, s, true);
            FG_CUDA(cudaMemsetAsync(fr->st_counts.p, 0, sizeof(uint32_t) * (P + 1), s));
            launch_frames_ball_count(v, p, P, fr->st_counts.as<uint32_t>(), s);
            scan_u32_to_u64(fr->st_counts.as<uint32_t>(), fr->st_offsets.as<uint64_t>(), static_cast<size_t>(P) + 1,
                            fr->st_scan.p, s);
        });
        uint64_t nb = 0;
        FG_CUDA(cudaMemcpyAsync(&nb, fr->st_offsets.as<uint64_t>() + P, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
        sync();
        if (nb >= (1ull << 32))
            runtime_error("a batched Steinhardt neighbour list holds fewer than 2^32 bonds");
        st->bond_hint = std::max<uint64_t>(st->bond_hint, nb);
        fr->st_j.alloc(sizeof(uint32_t) * std::max<uint64_t>(nb, 1));
        fr->st_vd.alloc(sizeof(float4) * std::max<uint64_t>(nb, 1));
        std::vector<uint64_t> key_b = outputs_key({g.id, nb, reinterpret_cast<uint64_t>(fr->st_offsets.p)});
        run_graph(fr->st_graph_b, fr->graphs, key_b, "graph:steinhardt_frames", [&] {
            launch_frames_ball_fill(v, p, P, fr->st_offsets.as<uint64_t>(), fr->st_j.as<uint32_t>(),
                                    fr->st_vd.as<float4>(), s);
            launch_segments_from_offsets(fr->st_counts.as<uint32_t>(), fr->st_offsets.as<uint64_t>(), P,
                                         fr->st_seg.as<uint32_t>(), s);
            enqueue_rest(static_cast<double>(nb) / std::max<uint32_t>(P, 1));
        });
        FG_CUDA(cudaGetLastError());
        FG_CUDA(cudaMemcpyAsync(sys.data(), fr->st_sys.p, sizeof(double) * sys.size(), cudaMemcpyDeviceToHost, s));
        sync();
    }
    st->order.assign(static_cast<size_t>(F) * st->st.nl, 0.0f);
    for (uint32_t f = 0; f < F; ++f)
        normalize_system(st, &sys[2 * static_cast<size_t>(f) * stride], &st->order[static_cast<size_t>(f) * st->st.nl]);
    st->computed = true;
}

fg_status fg_steinhardt_compute_frames(fg_steinhardt* st, fg_frames* fr, const fg_query_args* args)
{
    return guard([&] {
        require(st, "steinhardt");
        require(fr, "frames");
        require(args, "args");
        const fg_query_args a = batch_args(fr, args);
        steinhardt_frames(st, fr, a);
    });
}

fg_status fg_steinhardt_num_frames(const fg_steinhardt* st, uint32_t* out)
{
    return guard([&] {
        require(st, "steinhardt");
        require(out, "out");
        *out = st->frames;
    });
}

fg_status fg_batch_set_config(int shell, int warps_per_block, int hist_copies)
{
    return guard([&] {
        if (shell == 0)
        {
            g_forced = BatchHistConfig {0, 0, 0};
            return;
        }
        if (shell < 1 || shell > 2 || (warps_per_block != 4 && warps_per_block != 8) ||
            (hist_copies != 1 && hist_copies != 2 && hist_copies != warps_per_block))
            value_error("batch config: shell 1 or 2, 4 or 8 warps per block, 1, 2 or one per warp histogram copies");
        g_forced = BatchHistConfig {shell, warps_per_block, hist_copies};
    });
}

// ---------------------------------------------------------------------------
// Self-check of the box arithmetic's division (div_rn_recip) against IEEE division
// ---------------------------------------------------------------------------
namespace {
__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// Sample t: a divisor b (every other sample one of a few box lengths, else a
// random float in [2^-3, 2^13)) and a dividend a of either sign (random
// significand, exponent in [-10, 14)); counts quotients that differ in any bit
// from __fdiv_rn and keeps one offending pair.
__global__ void k_check_div(uint64_t n, uint64_t seed, unsigned long long* mism, float* example)
{
    const float lens[8] = {102.0f, 21.544f, 63.496f, 12.0f, 256.0f, 1.5874f, 3.0f, 7.0f};
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < n;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint64_t h = mix64(seed + t * 0x9e3779b97f4a7c15ull);
        float b;
        if (t & 1)
            b = lens[(h >> 40) & 7];
        else
            b = __uint_as_float(static_cast<uint32_t>(((124 + ((h >> 50) % 16)) << 23) | ((h >> 24) & 0x7fffff)));
        const uint32_t ea = 117 + static_cast<uint32_t>((h >> 10) % 24);
        const uint32_t sa = static_cast<uint32_t>(h & 1) << 31;
        const float a = __uint_as_float(sa | (ea << 23) | static_cast<uint32_t>((h >> 33) & 0x7fffff));
        const float q = div_rn_recip(a, b, __frcp_rn(b));
        const float r = __fdiv_rn(a, b);
        if (__float_as_uint(q) != __float_as_uint(r))
        {
            if (atomicAdd(mism, 1ull) == 0ull)
            {
                example[0] = a;
                example[1] = b;
            }
        }
    }
}
} // namespace

fg_status fg_check_division(uint64_t samples, uint64_t seed, uint64_t* mismatches, float* example)
{
    return guard([&] {
        require(mismatches, "mismatches");
        DevBuf buf;
        buf.alloc(sizeof(unsigned long long) + 2 * sizeof(float));
        cudaStream_t s = stream();
        FG_CUDA(cudaMemsetAsync(buf.p, 0, buf.bytes, s));
        auto* m = buf.as<unsigned long long>();
        auto* ex = reinterpret_cast<float*>(m + 1);
        if (samples > 0)
        {
            int dev = 0, sms = 152;
            FG_CUDA(cudaGetDevice(&dev));
            FG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            k_check_div<<<sms * 8, 256, 0, s>>>(samples, seed, m, ex);
            FG_CUDA(cudaGetLastError());
        }
        unsigned long long hm = 0;
        float hex[2] = {0.0f, 0.0f};
        FG_CUDA(cudaMemcpyAsync(&hm, m, sizeof(hm), cudaMemcpyDeviceToHost, s));
        FG_CUDA(cudaMemcpyAsync(hex, ex, sizeof(hex), cudaMemcpyDeviceToHost, s));
        sync();
        *mismatches = hm;
        if (example != nullptr)
        {
            example[0] = hex[0];
            example[1] = hex[1];
        }
    });
}

fg_status fg_set_count_kernel(int which)
{
    return guard([&] {
        if (which != 0 && which != 1)
            value_error("count kernel must be 0 (automatic) or 1 (block per cell, lanes over candidates)");
        g_count_kernel = which;
    });
}

fg_status fg_set_graphs(int enable)
{
    g_graphs_enabled = enable != 0;
    return FG_OK;
}

fg_status fg_autotune_report(char* buf, size_t len)
{
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (buf != nullptr && len > 0)
    {
        std::strncpy(buf, g_tune_log.c_str(), len - 1);
        buf[len - 1] = 0;
    }
    return g_tune_log.size() + 1 > len ? FG_ERR_VALUE : FG_OK;
}

} // extern "C"

namespace fg {

// Steinhardt of one (box, points) system with its own ball query (nlist ==
// NULL, AABB arithmetic, periodic box): the frames path with one frame. The
// reference sums each particle's bonds in query-iterator order here
// (Steinhardt.cc:136-147 with loopOverNeighborsIterator), not in NeighborList
// order, so no sorted list is built.
// RDF of one (box, points) system with its own ball query (nlist == NULL, the
// points as query points, AABB arithmetic, periodic box): the frames path with
// one frame - one grid build and the persistent histogram kernel with the
// autotuned launch shape. Returns false (caller takes the general path) otherwise.
bool rdf_ball_single(fg_rdf* rdf, fg_nq* nq, const float* dq, const fg_query_args* args)
{
    if (dq != nullptr || (nq->kind != FG_NQ_RAWPOINTS && nq->kind != FG_NQ_AABB) ||
        !(nq->box.periodic[0] && nq->box.periodic[1] && nq->box.periodic[2]))
        return false;
    fg_query_args a = *args;
    validate_args(a);
    if (a.mode != FG_MODE_BALL)
        return false;
    fg_frames fr;
    fr.graphs = false;
    fr.boxes.push_back(nq->box);
    fr.n.push_back(nq->n);
    fr.pt_base = {0u, nq->n};
    fr.total = nq->n;
    fr.dpts = nq->dpts;
    fr.d_pt_base.alloc(sizeof(uint32_t) * 2);
    FG_CUDA(cudaMemcpyAsync(fr.d_pt_base.p, fr.pt_base.data(), sizeof(uint32_t) * 2, cudaMemcpyHostToDevice, stream()));
    const fg_query_args checked = batch_args(&fr, &a);
    rdf_frames(rdf, &fr, checked);
    return true;
}

bool steinhardt_ball_single(fg_steinhardt* st, fg_nq* nq, const fg_query_args* args)
{
    if ((nq->kind != FG_NQ_RAWPOINTS && nq->kind != FG_NQ_AABB) ||
        !(nq->box.periodic[0] && nq->box.periodic[1] && nq->box.periodic[2]))
        return false;
    fg_query_args a = *args;
    validate_args(a);
    if (a.mode != FG_MODE_BALL)
        return false;
    fg_frames fr;
    fr.graphs = false;
    fr.boxes.push_back(nq->box);
    fr.n.push_back(nq->n);
    fr.pt_base = {0u, nq->n};
    fr.total = nq->n;
    fr.dpts = nq->dpts;
    fr.d_pt_base.alloc(sizeof(uint32_t) * 2);
    FG_CUDA(cudaMemcpyAsync(fr.d_pt_base.p, fr.pt_base.data(), sizeof(uint32_t) * 2, cudaMemcpyHostToDevice, stream()));
    const fg_query_args checked = batch_args(&fr, &a);
    steinhardt_frames(st, &fr, checked);
    return true;
}

} // namespace fg
