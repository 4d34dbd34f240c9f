// Steinhardt order parameters (freud/order/Steinhardt.cc:120-359).
//
// Layout: qlm for each l is an (N, 2l+1) complex64 array in the reference's m
// order 0..l, -1..-l (the particle_harmonics contract pinned by test_qlmi).
//
// k_qlm: LANES threads per particle, thread m (0 <= m <= max_l) owns +m and -m of
// every requested l. Per bond it recomputes the float32 pair vector as
// box.wrap(p_j - p_i) (Steinhardt.cc:155), takes cos(theta) = clamp(z/d) with the
// bond distance d (Steinhardt.cc:163-172) and e^{i phi} from (x, y), then runs the
// normalised associated-Legendre recurrence in l for its m entirely in registers:
//   Q_m^m     = K_m sin^m(theta)                       (K_m includes (-1)^m)
//   Q_{m+1}^m = sqrt(2m+3) x Q_m^m
//   Q_l^m     = a_lm (x Q_{l-1}^m - b_lm Q_{l-2}^m)
// so Y_l^m = Q_l^m e^{i m phi} and Y_l^{-m} = (-1)^m conj(Y_l^m), equal to
// scipy.special.sph_harm_y. Accumulates w * Y, divides by the total weight, and
// reduces ql over the particle's lanes with shuffles.
// k_ave: the same mapping gathers the neighbours' qlm (Steinhardt.cc:224-289).
// k_wl: thread per (particle, l), Wigner-3j triple sum with compensated float sum.
// k_sys: FP64 column sums of qlm (or averaged qlm) / N for the system order.
#include <cmath>
#include <cstdint>

#include "fg_common.cuh"
#include "fg_steinhardt.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__constant__ float c_K[ST_MAX_L + 1];                    // Q_m^m prefactors
__constant__ float c_a[(ST_MAX_L + 1) * (ST_MAX_L + 1)]; // a_lm at [l*(L+1)+m]
__constant__ float c_b[(ST_MAX_L + 1) * (ST_MAX_L + 1)]; // b_lm

template<int LANES>
__global__ void __launch_bounds__(128)
    k_qlm(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
          const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
          const uint32_t* __restrict__ cnt, const float* __restrict__ bvec, StLs ls, int weighted,
          float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES;               // m owned by this thread
    const int group = lane / LANES;             // particle slot within the warp
    const int groups_per_block = blockDim.x / LANES;
    const unsigned gmask = LANES == 32 ? FULL : (((1u << LANES) - 1u) << (group * LANES));
    const int m = sub;
    (void) group;
    for (uint32_t i = blockIdx.x * groups_per_block + threadIdx.x / LANES; i < n; i += gridDim.x * groups_per_block)
    {
        const bool live = true;
        float acc_re[ST_MAX_NL][2];
        float acc_im[ST_MAX_NL][2];
#pragma unroll
        for (int k = 0; k < ST_MAX_NL; ++k)
        {
            acc_re[k][0] = acc_re[k][1] = acc_im[k][0] = acc_im[k][1] = 0.0f;
        }
        float tw = 0.0f;
        if (live && m <= ls.max_l)
        {
            const float pix = pts[3 * (size_t) i];
            const float piy = pts[3 * (size_t) i + 1];
            const float piz = pts[3 * (size_t) i + 2];
            const uint32_t b0 = seg[i];
            const uint32_t b1 = b0 + cnt[i];
            for (uint32_t e = b0; e < b1; ++e)
            {
                float dx, dy, dz;
                if (bvec != nullptr)
                {
                    dx = bvec[3 * (size_t) e];
                    dy = bvec[3 * (size_t) e + 1];
                    dz = bvec[3 * (size_t) e + 2];
                }
                else
                {
                    const uint32_t j = ij[e].y;
                    box_wrap(b, __fsub_rn(pts[3 * (size_t) j], pix), __fsub_rn(pts[3 * (size_t) j + 1], piy),
                             __fsub_rn(pts[3 * (size_t) j + 2], piz), dx, dy, dz);
                }
                const float w = weighted ? weights[e] : 1.0f;
                const float d = dist[e];
                float ct = d == 0.0f ? 1.0f : fminf(1.0f, fmaxf(-1.0f, dz / d));
                const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
                const float rho = sqrtf(dx * dx + dy * dy);
                float cp = 1.0f, sp = 0.0f;
                if (rho > 0.0f)
                {
                    cp = dx / rho;
                    sp = dy / rho;
                }
                // e^{i m phi} and sin^m(theta)
                float em_re = 1.0f, em_im = 0.0f, sm = 1.0f;
                for (int t = 0; t < m; ++t)
                {
                    const float nr = em_re * cp - em_im * sp;
                    em_im = em_re * sp + em_im * cp;
                    em_re = nr;
                    sm *= st;
                }
                float q_lm2 = 0.0f;
                float q_lm1 = c_K[m] * sm; // Q_m^m
                // advance over the requested ls (ascending) while running the recurrence in l
                for (int l = m; l <= ls.max_l; ++l)
                {
                    float q;
                    if (l == m)
                    {
                        q = q_lm1;
                    }
                    else if (l == m + 1)
                    {
                        q = sqrtf(2.0f * m + 3.0f) * ct * q_lm1;
                        q_lm2 = q_lm1;
                        q_lm1 = q;
                    }
                    else
                    {
                        q = c_a[l * (ST_MAX_L + 1) + m] * (ct * q_lm1 - c_b[l * (ST_MAX_L + 1) + m] * q_lm2);
                        q_lm2 = q_lm1;
                        q_lm1 = q;
                    }
#pragma unroll
                    for (int k = 0; k < ST_MAX_NL; ++k)
                    {
                        if (k < ls.nl && ls.l[k] == l)
                        {
                            const float yr = w * q * em_re;
                            const float yi = w * q * em_im;
                            acc_re[k][0] += yr;
                            acc_im[k][0] += yi;
                            // Y_l^{-m} = (-1)^m conj(Y_l^m)
                            const float sgn = (m & 1) ? -1.0f : 1.0f;
                            acc_re[k][1] += sgn * yr;
                            acc_im[k][1] -= sgn * yi;
                        }
                    }
                }
                tw += w;
            }
        }
        // normalise, write, and reduce ql over the particle's lanes
#pragma unroll
        for (int k = 0; k < ST_MAX_NL; ++k)
        {
            if (k >= ls.nl)
            {
                break;
            }
            const int l = ls.l[k];
            float part = 0.0f;
            if (live && m <= l)
            {
                const float qr = acc_re[k][0] / tw;
                const float qi = acc_im[k][0] / tw;
                float2* row = qlm_out + ls.qlm_offset[k] + static_cast<size_t>(i) * (2 * l + 1);
                row[m] = make_float2(qr, qi);
                part = qr * qr + qi * qi;
                if (m > 0)
                {
                    const float nr = acc_re[k][1] / tw;
                    const float ni = acc_im[k][1] / tw;
                    row[l + m] = make_float2(nr, ni);
                    part += nr * nr + ni * ni;
                }
            }
            for (int o = LANES / 2; o > 0; o >>= 1)
            {
                part += __shfl_xor_sync(gmask, part, o, LANES);
            }
            if (live && sub == 0)
            {
                ql_out[static_cast<size_t>(i) * ls.nl + k] = sqrtf(part * ls.norm[k]);
            }
        }
    }
}

// Neighbour averaging: ave(i) = (sum_j qlm(j) + qlm(i)) / (1 + n_i).
template<int LANES>
__global__ void __launch_bounds__(128)
    k_ave(uint32_t n, const uint2* __restrict__ ij, const uint32_t* __restrict__ seg, const uint32_t* __restrict__ cnt,
          StLs ls, const float2* __restrict__ qlm, float2* __restrict__ ave, float* __restrict__ ql_ave)
{
    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES;
    const int group = lane / LANES;
    const int groups_per_block = blockDim.x / LANES;
    const unsigned gmask = LANES == 32 ? FULL : (((1u << LANES) - 1u) << (group * LANES));
    const int m = sub;
    (void) group;
    for (uint32_t i = blockIdx.x * groups_per_block + threadIdx.x / LANES; i < n; i += gridDim.x * groups_per_block)
    {
        const bool live = true;
        const uint32_t b0 = live ? seg[i] : 0;
        const uint32_t b1 = live ? b0 + cnt[i] : 0;
#pragma unroll
        for (int k = 0; k < ST_MAX_NL; ++k)
        {
            if (k >= ls.nl)
            {
                break;
            }
            const int l = ls.l[k];
            float part = 0.0f;
            if (live && m <= l)
            {
                const float2* base = qlm + ls.qlm_offset[k];
                float pr = 0.f, pim = 0.f, nr = 0.f, nim = 0.f;
                for (uint32_t e = b0; e < b1; ++e)
                {
                    const float2* rj = base + static_cast<size_t>(ij[e].y) * (2 * l + 1);
                    const float2 a = rj[m];
                    pr += a.x;
                    pim += a.y;
                    if (m > 0)
                    {
                        const float2 c = rj[l + m];
                        nr += c.x;
                        nim += c.y;
                    }
                }
                const float2* ri = base + static_cast<size_t>(i) * (2 * l + 1);
                const float cntf = static_cast<float>(1u + (b1 - b0));
                const float2 a = ri[m];
                pr = (pr + a.x) / cntf;
                pim = (pim + a.y) / cntf;
                float2* out = ave + ls.qlm_offset[k] + static_cast<size_t>(i) * (2 * l + 1);
                out[m] = make_float2(pr, pim);
                part = pr * pr + pim * pim;
                if (m > 0)
                {
                    const float2 c = ri[l + m];
                    nr = (nr + c.x) / cntf;
                    nim = (nim + c.y) / cntf;
                    out[l + m] = make_float2(nr, nim);
                    part += nr * nr + nim * nim;
                }
            }
            for (int o = LANES / 2; o > 0; o >>= 1)
            {
                part += __shfl_xor_sync(gmask, part, o, LANES);
            }
            if (live && sub == 0)
            {
                ql_ave[static_cast<size_t>(i) * ls.nl + k] = sqrtf(part * ls.norm[k]);
            }
        }
    }
}

// Wl per (particle, l): sum over m1 + m2 + m3 = 0 of w3j * Re(q_m1 q_m2 q_m3)
// (Wigner3j.cc:22-57), coefficients in the reference's iteration order.
__global__ void __launch_bounds__(128)
    k_wl(uint32_t n, int l, int k, int nl, size_t qlm_offset, const float2* __restrict__ src,
         const float* __restrict__ w3j, const float* __restrict__ qnorm, int normalize, float norm_factor,
         float* __restrict__ wl_out)
{
    extern __shared__ float2 rows[];
    const int nm = 2 * l + 1;
    const uint32_t i0 = blockIdx.x * blockDim.x;
    // stage the block's rows (coalesced)
    for (uint32_t e = threadIdx.x; e < blockDim.x * static_cast<uint32_t>(nm); e += blockDim.x)
    {
        const uint32_t gi = i0 + e / nm;
        rows[e] = gi < n ? src[qlm_offset + static_cast<size_t>(i0) * nm + e] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const uint32_t i = i0 + threadIdx.x;
    if (i >= n)
    {
        return;
    }
    const float2* q = rows + threadIdx.x * nm;
    float sum = 0.0f, comp = 0.0f;
    int c = 0;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        const float2 a = q[m1 < 0 ? l - m1 : m1];
        const int lo = max(-l - m1, -l);
        const int hi = min(l - m1, l);
        for (int m2 = lo; m2 <= hi; ++m2, ++c)
        {
            const int m3 = -m1 - m2;
            const float2 bq = q[m2 < 0 ? l - m2 : m2];
            const float2 cq = q[m3 < 0 ? l - m3 : m3];
            const float abr = a.x * bq.x - a.y * bq.y;
            const float abi = a.x * bq.y + a.y * bq.x;
            const float term = w3j[c] * (abr * cq.x - abi * cq.y);
            // compensated (Kahan) summation
            const float y = term - comp;
            const float t = sum + y;
            comp = (t - sum) - y;
            sum = t;
        }
    }
    if (normalize)
    {
        const float nf = sqrtf(norm_factor) / qnorm[static_cast<size_t>(i) * nl + k];
        sum *= nf * nf * nf;
    }
    wl_out[static_cast<size_t>(i) * nl + k] = sum;
}

// FP64 column sums: sys[c] += sum_i src[i, c] / n over a row range, compensated.
__global__ void k_sys(uint32_t n, int ncols, size_t offset, const float2* __restrict__ src, double* sys)
{
    const int c = threadIdx.x;
    if (c >= ncols)
    {
        return;
    }
    const uint32_t rows_per_block = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t r0 = blockIdx.x * rows_per_block;
    const uint32_t r1 = min(n, r0 + rows_per_block);
    double sr = 0.0, si = 0.0, cr = 0.0, ci = 0.0;
    for (uint32_t r = r0; r < r1; ++r)
    {
        const float2 v = src[offset + static_cast<size_t>(r) * ncols + c];
        const double yr = static_cast<double>(v.x) / n - cr;
        const double tr = sr + yr;
        cr = (tr - sr) - yr;
        sr = tr;
        const double yi = static_cast<double>(v.y) / n - ci;
        const double ti = si + yi;
        ci = (ti - si) - yi;
        si = ti;
    }
    if (r1 > r0)
    {
        atomicAdd(&sys[2 * c], sr);
        atomicAdd(&sys[2 * c + 1], si);
    }
}

int sm_count()
{
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms;
}

} // namespace

void st_upload_tables(cudaStream_t s)
{
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && done[dev])
    {
        return;
    }
    const int L = ST_MAX_L;
    float K[ST_MAX_L + 1];
    static float A[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    static float B[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    for (int m = 0; m <= L; ++m)
    {
        // K_m = (-1)^m (2m-1)!! sqrt((2m+1) / (4 pi (2m)!)), in log space
        double lg = 0.5 * (std::log(2.0 * m + 1.0) - std::log(4.0 * M_PI) - std::lgamma(2.0 * m + 1.0));
        for (int t = 1; t <= m; ++t)
        {
            lg += std::log(2.0 * t - 1.0);
        }
        K[m] = static_cast<float>(((m & 1) ? -1.0 : 1.0) * std::exp(lg));
        for (int l = 0; l <= L; ++l)
        {
            double a = 0.0, bb = 0.0;
            if (l >= m + 2)
            {
                a = std::sqrt((4.0 * l * l - 1.0) / (static_cast<double>(l) * l - static_cast<double>(m) * m));
                bb = std::sqrt(((l - 1.0) * (l - 1.0) - static_cast<double>(m) * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
            }
            A[l * (L + 1) + m] = static_cast<float>(a);
            B[l * (L + 1) + m] = static_cast<float>(bb);
        }
    }
    cudaMemcpyToSymbolAsync(c_K, K, sizeof(K), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_a, A, sizeof(A), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_b, B, sizeof(B), 0, cudaMemcpyHostToDevice, s);
    cudaStreamSynchronize(s);
    if (dev < 64)
    {
        done[dev] = true;
    }
}

static int lanes_for(int max_l)
{
    return max_l < 8 ? 8 : (max_l < 16 ? 16 : 32);
}

void launch_qlm(const DevBox& box, const float* pts, uint32_t n, const uint2* ij, const float* dist,
                const float* weights, const uint32_t* seg, const uint32_t* cnt, const StLs& ls, int weighted,
                float2* qlm, float* ql, cudaStream_t s, const float* bond_vec)
{
    if (n == 0)
    {
        return;
    }
    const int lanes = lanes_for(ls.max_l);
    const uint32_t groups = 128 / lanes;
    uint32_t blocks = (n + groups - 1) / groups;
    const uint32_t cap = static_cast<uint32_t>(sm_count()) * 16;
    blocks = blocks < cap ? blocks : cap;
    if (lanes == 8)
        {
            ProfScope prof_("k_qlm<8>", s);
            k_qlm<8><<<blocks, 128, 0, s>>>(box, pts, n, ij, dist, weights, seg, cnt, bond_vec, ls, weighted, qlm, ql);
        }
    else if (lanes == 16)
        {
            ProfScope prof_("k_qlm<16>", s);
            k_qlm<16><<<blocks, 128, 0, s>>>(box, pts, n, ij, dist, weights, seg, cnt, bond_vec, ls, weighted, qlm, ql);
        }
    else
        {
            ProfScope prof_("k_qlm<32>", s);
            k_qlm<32><<<blocks, 128, 0, s>>>(box, pts, n, ij, dist, weights, seg, cnt, bond_vec, ls, weighted, qlm, ql);
        }
}

void launch_ave(uint32_t n, const uint2* ij, const uint32_t* seg, const uint32_t* cnt, const StLs& ls,
                const float2* qlm, float2* ave, float* ql_ave, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    const int lanes = lanes_for(ls.max_l);
    const uint32_t groups = 128 / lanes;
    uint32_t blocks = (n + groups - 1) / groups;
    const uint32_t cap = static_cast<uint32_t>(sm_count()) * 16;
    blocks = blocks < cap ? blocks : cap;
    if (lanes == 8)
        {
            ProfScope prof_("k_ave<8>", s);
            k_ave<8><<<blocks, 128, 0, s>>>(n, ij, seg, cnt, ls, qlm, ave, ql_ave);
        }
    else if (lanes == 16)
        {
            ProfScope prof_("k_ave<16>", s);
            k_ave<16><<<blocks, 128, 0, s>>>(n, ij, seg, cnt, ls, qlm, ave, ql_ave);
        }
    else
        {
            ProfScope prof_("k_ave<32>", s);
            k_ave<32><<<blocks, 128, 0, s>>>(n, ij, seg, cnt, ls, qlm, ave, ql_ave);
        }
}

void launch_wl(uint32_t n, const StLs& ls, int k, const float2* src, const float* w3j_dev, const float* qnorm,
               int normalize, float* wl, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    const int l = ls.l[k];
    const size_t smem = 128 * static_cast<size_t>(2 * l + 1) * sizeof(float2);
    static bool configured = false;
    if (!configured)
    {
        cudaFuncSetAttribute(k_wl, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(128 * (2 * ST_MAX_L + 1) * sizeof(float2)));
        configured = true;
    }
    {
        ProfScope prof_("k_wl", s);
        k_wl<<<(n + 127) / 128, 128, smem, s>>>(n, l, k, ls.nl, ls.qlm_offset[k], src, w3j_dev, qnorm, normalize,
                                                ls.norm[k], wl);
    }
}

void launch_sys(uint32_t n, const StLs& ls, const float2* src, double* sys, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    size_t col_off = 0;
    for (int k = 0; k < ls.nl; ++k)
    {
        const int nm = 2 * ls.l[k] + 1;
        const uint32_t blocks = static_cast<uint32_t>(sm_count()) * 4;
        {
            ProfScope prof_("k_sys", s);
            k_sys<<<blocks, 64, 0, s>>>(n, nm, ls.qlm_offset[k], src, sys + 2 * col_off);
        }
        col_off += nm;
    }
}

} // namespace fg
