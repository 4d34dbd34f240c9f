// Ball queries, block per home cell, warp per query with compacted exact tests.
//
// A block takes one cell of the query grid and stages the candidate set shared by
// all of its queries - the points of the 27 (9 in 2D) neighbouring cells, each
// with its cell wrap - in shared memory once. Each warp then takes one query of
// the cell at a time and scans the staged candidates 32 per step.
//
// Pair arithmetic is exact and identical to the warp-per-query kernels
// (AABBQuery.cc:93,125 / LinkCell.cc:522). In wrap arithmetic the exact
// box.wrap (three IEEE divisions) is expensive, so a cheap prefilter on the
// cell-shifted positions classifies each candidate as certainly outside
// (> r_max + delta), certainly inside (< r_max - delta) or undecided. Candidates
// that need the exact test are appended to a per-warp queue in scan order and
// tested 32 at a time, so the exact arithmetic runs with full lanes. The
// prefilter is only enabled when every periodic axis has >= 3 cells and
// r_max + delta is below half the smallest plane distance, where the
// cell-derived image is the minimum image of every possible bond.
//
// COUNT: bonds per query (candidates certainly inside need no exact test).
// EMIT:  the staged candidates are sorted by point index once per cell, so the
//        queue - and hence each query's accepted bonds - comes out in the
//        reference's (i, j) order (NeighborBond.h:80-95); bonds are written at the
//        query's offset as they are accepted, 32 consecutive slots at a time.
// HIST:  fused RDF binning (RDF.cc:101-110, Histogram.h:152-174).
// Cells whose candidate set exceeds the shared-memory capacity hand their queries
// to the warp-per-query kernels.
#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int CWARPS = 8;
constexpr int CTHREADS = CWARPS * 32;
constexpr int CAP = 2048; // staged candidates per cell
constexpr int HIST_BINS_SMEM = 4096;

enum CellMode
{
    CM_COUNT = 0,
    CM_EMIT = 1,
    CM_HIST = 2,
};

__device__ __forceinline__ int img_ax(int bits, int axis)
{
    return static_cast<int>(static_cast<int8_t>((bits >> (8 * axis)) & 0xff));
}

struct CellShared
{
    float4 pos[CAP];             // x, y, z, packed integer box image
    float4 ps[CAP];              // prefilter position (wrap arithmetic)
    uint32_t j[CAP];             // point index
    unsigned char wrap[CAP];     // cell wrap code (wx+1) + 3(wy+1) + 9(wz+1)
    unsigned long long key[CAP]; // (j << 32) | slot, sorted per cell (EMIT)
    unsigned short queue[CWARPS][64];
    uint32_t item_start[32];
    uint32_t item_off[33];
    int item_wrap[32];
    float img[27][3];
    uint32_t total;
    unsigned int hist[HIST_BINS_SMEM];
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

template<int MODE>
__global__ void __launch_bounds__(CTHREADS, 2)
    k_cell(DevBox b, DevGrid g, DevGrid qg, BallParams p, float pre_out2, float pre_in2,
           uint32_t* __restrict__ counts, const uint64_t* __restrict__ offsets, uint2* __restrict__ ij,
           float* __restrict__ dist, float* __restrict__ vec, uint32_t* overflow, uint32_t* overflow_n, HistParams h,
           unsigned long long* __restrict__ hist)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CellShared& S = *reinterpret_cast<CellShared*>(smem_raw);
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    const int warp = tid >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const bool use_pre = pre_out2 > 0.0f;
    const bool smem_hist = MODE == CM_HIST && h.bins <= HIST_BINS_SMEM;
    unsigned short* queue = S.queue[warp];

    for (int t = tid; t < 81; t += CTHREADS)
    {
        S.img[t / 3][t % 3] = b.img[t / 3][t % 3];
    }
    if (MODE == CM_HIST && smem_hist)
    {
        for (int t = tid; t < static_cast<int>(h.bins); t += CTHREADS)
        {
            S.hist[t] = 0;
        }
    }
    __syncthreads();

    for (int c = blockIdx.x; c < qg.ncell; c += gridDim.x)
    {
        const uint32_t q0 = qg.start[c];
        const uint32_t nqc = qg.start[c + 1] - q0;
        if (nqc == 0)
        {
            continue;
        }
        const int cz = c / (g.dim[0] * g.dim[1]);
        const int cy = (c / g.dim[0]) % g.dim[1];
        const int cx = c % g.dim[0];
        // ---- stencil items and their offsets (warp 0) ----
        if (warp == 0)
        {
            uint32_t cnt = 0, st = 0;
            int wr = 13;
            const int nst = b.is2d ? 9 : 27;
            if (lane < nst)
            {
                const int dx = lane % 3 - 1;
                const int dy = (lane / 3) % 3 - 1;
                const int dz = b.is2d ? 0 : lane / 9 - 1;
                auto ok = [&](int d, int dim) {
                    if (p.arith == ARITH_AABB || dim >= 3)
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
            S.item_start[lane] = st;
            S.item_off[lane] = incl - cnt;
            S.item_wrap[lane] = wr;
            if (lane == 31)
            {
                S.item_off[32] = incl;
                S.total = incl;
            }
        }
        __syncthreads();
        const uint32_t T = S.total;
        if (T > CAP)
        {
            // hand this cell's queries to the warp-per-query kernel
            for (uint32_t k = tid; k < nqc; k += CTHREADS)
            {
                overflow[atomicAdd(overflow_n, 1u)] = q0 + k;
            }
            __syncthreads();
            continue;
        }
        // ---- stage candidates ----
        for (uint32_t t = tid; t < T; t += CTHREADS)
        {
            int s = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1)
            {
                if (s + step < 32 && S.item_off[s + step] <= t)
                    s += step;
            }
            const uint32_t slot = S.item_start[s] + (t - S.item_off[s]);
            const float4 pp = g.cpos[slot];
            const int wr = S.item_wrap[s];
            const uint32_t jj = g.cidx[slot];
            S.pos[t] = pp;
            S.j[t] = jj;
            S.wrap[t] = static_cast<unsigned char>(wr);
            if (use_pre)
            {
                const int pim = __float_as_int(pp.w);
                const float3 sp = shifted(b, pp, (wr % 3 - 1) - img_ax(pim, 0), ((wr / 3) % 3 - 1) - img_ax(pim, 1),
                                          (wr / 9 - 1) - img_ax(pim, 2));
                S.ps[t] = make_float4(sp.x, sp.y, sp.z, 0.0f);
            }
            if (MODE == CM_EMIT)
            {
                S.key[t] = (static_cast<unsigned long long>(jj) << 32) | t;
            }
        }
        if (MODE == CM_EMIT)
        {
            uint32_t np2 = 32;
            while (np2 < T)
                np2 <<= 1;
            for (uint32_t t = T + tid; t < np2; t += CTHREADS)
                S.key[t] = ~0ull;
            __syncthreads();
            // bitonic sort of the staged candidates by point index
            for (uint32_t k = 2; k <= np2; k <<= 1)
            {
                for (uint32_t jj = k >> 1; jj > 0; jj >>= 1)
                {
                    for (uint32_t e = tid; e < np2 / 2; e += CTHREADS)
                    {
                        // e indexes compare-exchange pairs: lower element of pair e
                        const uint32_t lo = ((e & ~(jj - 1)) << 1) | (e & (jj - 1));
                        const uint32_t hi = lo | jj;
                        const bool up = (lo & k) == 0;
                        const unsigned long long a = S.key[lo], cc = S.key[hi];
                        if ((a > cc) == up)
                        {
                            S.key[lo] = cc;
                            S.key[hi] = a;
                        }
                    }
                    __syncthreads();
                }
            }
        }
        __syncthreads();

        // ---- warp per query ----
        const uint32_t nchunks = (T + 31) / 32;
        for (uint32_t qq = warp; qq < nqc; qq += CWARPS)
        {
            const float4 q = qg.cpos[q0 + qq];
            const uint32_t qi = qg.cidx[q0 + qq];
            const int qimg = __float_as_int(q.w);
            const float3 qs = use_pre ? shifted(b, q, -img_ax(qimg, 0), -img_ax(qimg, 1), -img_ax(qimg, 2))
                                      : make_float3(0.f, 0.f, 0.f);
            uint32_t count = 0;
            uint32_t qn = 0;
            uint64_t out = MODE == CM_EMIT ? offsets[qi] : 0;

            // exact test of the first n queued candidates (n <= 32), in queue order
            auto process = [&](uint32_t n) {
                bool acc = false;
                float rx = 0.f, ry = 0.f, rz = 0.f, rsq = 0.f;
                uint32_t t = 0;
                if (lane < static_cast<int>(n))
                {
                    t = queue[lane];
                    if (MODE == CM_EMIT)
                        t = static_cast<uint32_t>(S.key[t] & 0xffffffffull);
                    if (exact_vec(b, S.img, p.arith, q, qimg, S.pos[t], S.wrap[t], rx, ry, rz))
                    {
                        rsq = dot3(rx, ry, rz);
                        acc = rsq < p.r_max_sq && rsq >= p.r_min_sq;
                    }
                }
                const unsigned am = __ballot_sync(FULL, acc);
                if (MODE == CM_EMIT)
                {
                    if (acc)
                    {
                        const uint64_t o = out + count + __popc(am & lt);
                        ij[o] = make_uint2(qi, S.j[t]);
                        dist[o] = __fsqrt_rn(rsq);
                        vec[3 * o] = rx;
                        vec[3 * o + 1] = ry;
                        vec[3 * o + 2] = rz;
                    }
                }
                else if (MODE == CM_HIST)
                {
                    if (acc)
                    {
                        const float d = __fsqrt_rn(rsq);
                        if (!(d < h.h_min || d >= h.h_max))
                        {
                            uint32_t bin = static_cast<uint32_t>(__fmul_rn(__fsub_rn(d, h.h_min), h.h_inv));
                            if (bin == h.bins)
                                bin = h.bins - 1;
                            if (smem_hist)
                                atomicAdd(&S.hist[bin], 1u);
                            else
                                atomicAdd(&hist[bin], 1ull);
                        }
                    }
                }
                count += __popc(am);
            };

            for (uint32_t ch = 0; ch < nchunks; ++ch)
            {
                const uint32_t e = ch * 32 + lane;
                const bool live = e < T;
                bool need = false;
                bool inside = false;
                if (live)
                {
                    const uint32_t t = MODE == CM_EMIT ? static_cast<uint32_t>(S.key[e] & 0xffffffffull) : e;
                    if (!(p.exclude_ii && S.j[t] == qi))
                    {
                        if (use_pre)
                        {
                            const float4 ps = S.ps[t];
                            const float dx = ps.x - qs.x, dy = ps.y - qs.y, dz = ps.z - qs.z;
                            const float d2 = dx * dx + dy * dy + dz * dz;
                            if (MODE == CM_COUNT && d2 < pre_in2)
                                inside = true;
                            else
                                need = d2 <= pre_out2;
                        }
                        else
                        {
                            need = true;
                        }
                    }
                }
                if (MODE == CM_COUNT)
                {
                    count += __popc(__ballot_sync(FULL, inside));
                }
                const unsigned nm = __ballot_sync(FULL, need);
                if (need)
                {
                    queue[qn + __popc(nm & lt)] = static_cast<unsigned short>(e);
                }
                qn += __popc(nm);
                __syncwarp();
                if (qn >= 32)
                {
                    process(32);
                    // move the remaining entries to the front of the queue
                    const uint32_t rest = qn - 32;
                    unsigned short v = 0;
                    if (lane < static_cast<int>(rest))
                        v = queue[32 + lane];
                    __syncwarp();
                    if (lane < static_cast<int>(rest))
                        queue[lane] = v;
                    __syncwarp();
                    qn = rest;
                }
            }
            if (qn > 0)
            {
                process(qn);
                __syncwarp();
            }
            if (MODE == CM_COUNT && lane == 0)
            {
                counts[qi] = count;
            }
        }
        __syncthreads();
    }
    if (MODE == CM_HIST && smem_hist)
    {
        __syncthreads();
        for (int bin = tid; bin < static_cast<int>(h.bins); bin += CTHREADS)
        {
            if (S.hist[bin] != 0)
                atomicAdd(&hist[bin], static_cast<unsigned long long>(S.hist[bin]));
        }
    }
}

int cell_blocks(int ncell)
{
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int want = 2 * sms;
    return ncell < want ? (ncell < 1 ? 1 : ncell) : want;
}

template<int MODE> void configure()
{
    static bool done = false;
    if (!done)
    {
        cudaFuncSetAttribute(k_cell<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(sizeof(CellShared)));
        done = true;
    }
}

} // namespace

size_t cell_smem_bytes()
{
    return sizeof(CellShared);
}

void launch_cell(int mode, const DevBox& box, const DevGrid& g, const DevGrid& qg, const BallParams& p, float pre_out2,
                 float pre_in2, uint32_t* counts, const uint64_t* offsets, uint2* ij, float* dist, float* vec,
                 uint32_t* overflow, uint32_t* overflow_n, const HistParams& h, unsigned long long* hist,
                 cudaStream_t s)
{
    const int blocks = cell_blocks(qg.ncell);
    const size_t smem = sizeof(CellShared);
    if (mode == CM_COUNT)
    {
        configure<CM_COUNT>();
        ProfScope prof_("k_cell<COUNT>", s);
        k_cell<CM_COUNT><<<blocks, CTHREADS, smem, s>>>(box, g, qg, p, pre_out2, pre_in2, counts, offsets, ij, dist,
                                                         vec, overflow, overflow_n, h, hist);
    }
    else if (mode == CM_EMIT)
    {
        configure<CM_EMIT>();
        ProfScope prof_("k_cell<EMIT>", s);
        k_cell<CM_EMIT><<<blocks, CTHREADS, smem, s>>>(box, g, qg, p, pre_out2, pre_in2, counts, offsets, ij, dist, vec,
                                                        overflow, overflow_n, h, hist);
    }
    else
    {
        configure<CM_HIST>();
        ProfScope prof_("k_cell<HIST>", s);
        k_cell<CM_HIST><<<blocks, CTHREADS, smem, s>>>(box, g, qg, p, pre_out2, pre_in2, counts, offsets, ij, dist, vec,
                                                        overflow, overflow_n, h, hist);
    }
}

} // namespace fg
