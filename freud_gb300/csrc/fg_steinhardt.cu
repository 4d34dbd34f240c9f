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
// The FP64 system sums (qlm or averaged qlm over the particles, divided by N)
// are taken by the per-frame column-sum kernels of fg_batch.cu.
#include <algorithm>
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

// cos(theta) = clamp(dz / d) and sin(theta) of a bond (Steinhardt.cc:163-172: the
// wrapped z over the bond distance, clamped; theta = 0 when d = 0). cos rounded
// to float loses sin near the poles, where 1 - cos^2 cancels; the quotient's
// residual lo = (dz - hi d) / d (the remainder is exact through an FMA) makes
// 1 - cos^2 = (1 - hi^2) - 2 hi lo, each product fused, so sin(theta) is accurate
// to about one ulp at every angle, as FP64 gives it.
__device__ __forceinline__ void bond_angle(float dz, float d, float& ct, float& st)
{
    ct = 1.0f;
    st = 0.0f;
    if (d == 0.0f)
        return;
    const float hi = dz / d;
    const float lo = __fmaf_rn(-hi, d, dz) / d;
    if (hi > 1.0f || (hi == 1.0f && lo >= 0.0f))
        return;
    if (hi < -1.0f || (hi == -1.0f && lo <= 0.0f))
    {
        ct = -1.0f;
        return;
    }
    ct = hi;
    st = sqrtf(fmaxf(0.0f, __fmaf_rn(-2.0f * hi, lo, __fmaf_rn(-hi, hi, 1.0f))));
}

// LANES threads per particle; thread a owns the orders ma = a and mb = l_max - a
// (when mb > ma), so the two normalised Legendre recurrences of a thread take
// l_max steps together and no thread of the group waits on another.
template<int LANES, int NL>
__global__ void __launch_bounds__(128)
    k_qlm(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
          const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
          const uint32_t* __restrict__ cnt, const float4* __restrict__ bvd, StLs ls, int weighted,
          float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    // recurrence coefficients staged once per block (threads read different m)
    __shared__ float s_a[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    __shared__ float s_b[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    __shared__ float s_K[ST_MAX_L + 1];
    for (int t = threadIdx.x; t <= ls.max_l * (ST_MAX_L + 1) + ST_MAX_L; t += blockDim.x)
    {
        s_a[t] = c_a[t];
        s_b[t] = c_b[t];
    }
    for (int t = threadIdx.x; t <= ST_MAX_L; t += blockDim.x)
        s_K[t] = c_K[t];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES;
    const int group = lane / LANES;             // particle slot within the warp
    const int groups_per_block = blockDim.x / LANES;
    const unsigned gmask = LANES == 32 ? FULL : (((1u << LANES) - 1u) << (group * LANES));
    const int lmax = ls.max_l;
    const int used = lmax / 2 + 1;              // threads with an order of their own
    const bool has_a = sub < used;
    const int ma = has_a ? sub : 0;             // idle threads shadow thread 0, with zero weight
    const int mb = lmax - ma;
    const bool has_b = has_a && mb > ma;
    const int split = lmax - ma;                // steps of the ma recurrence; the mb one takes ma steps
    const float ka = has_a ? s_K[ma] : 0.0f;
    const float kb = has_b ? s_K[mb] : 0.0f;
    const float c1a = sqrtf(2.0f * ma + 3.0f);
    const float c1b = sqrtf(2.0f * mb + 3.0f);
    const float sga = (ma & 1) ? -1.0f : 1.0f;
    const float sgb = (mb & 1) ? -1.0f : 1.0f;
    // slot kk holds the kk-th smallest requested l
    int lt[NL];
#pragma unroll
    for (int kk = 0; kk < NL; ++kk)
        lt[kk] = kk < ls.nl ? ls.l[ls.sorted_k[kk]] : -1;
    for (uint32_t i = blockIdx.x * groups_per_block + threadIdx.x / LANES; i < n; i += gridDim.x * groups_per_block)
    {
        float accA_re[NL][2], accA_im[NL][2], accB_re[NL][2], accB_im[NL][2];
#pragma unroll
        for (int k = 0; k < NL; ++k)
        {
            accA_re[k][0] = accA_re[k][1] = accA_im[k][0] = accA_im[k][1] = 0.0f;
            accB_re[k][0] = accB_re[k][1] = accB_im[k][0] = accB_im[k][1] = 0.0f;
        }
        float tw = 0.0f;
        const uint32_t b0 = seg[i];
        const uint32_t nbond = cnt[i];
        float pix = 0.f, piy = 0.f, piz = 0.f;
        if (bvd == nullptr)
        {
            pix = pts[3 * (size_t) i];
            piy = pts[3 * (size_t) i + 1];
            piz = pts[3 * (size_t) i + 2];
        }
        // bonds in batches of LANES: thread t computes the geometry of bond base + t
        // (independent loads in flight), then the group walks the batch with shuffles
        for (uint32_t base = 0; base < nbond; base += LANES)
        {
            float g_ct = 1.0f, g_st = 0.0f, g_cp = 1.0f, g_sp = 0.0f, g_w = 0.0f;
            if (base + sub < nbond)
            {
                const uint32_t e = b0 + base + sub;
                float dx, dy, dz, d;
                if (bvd != nullptr)
                {
                    const float4 v = bvd[e];
                    dx = v.x;
                    dy = v.y;
                    dz = v.z;
                    d = v.w;
                }
                else
                {
                    const uint32_t j = ij[e].y;
                    box_wrap(b, __fsub_rn(pts[3 * (size_t) j], pix), __fsub_rn(pts[3 * (size_t) j + 1], piy),
                             __fsub_rn(pts[3 * (size_t) j + 2], piz), dx, dy, dz);
                    d = dist[e];
                }
                g_w = weighted ? weights[e] : 1.0f;
                bond_angle(dz, d, g_ct, g_st);
                const float rho = sqrtf(dx * dx + dy * dy);
                if (rho > 0.0f)
                {
                    g_cp = dx / rho;
                    g_sp = dy / rho;
                }
            }
            const uint32_t nb_here = min(static_cast<uint32_t>(LANES), nbond - base);
            for (uint32_t t = 0; t < nb_here; ++t)
            {
                const float ct = __shfl_sync(gmask, g_ct, t, LANES);
                const float st = __shfl_sync(gmask, g_st, t, LANES);
                const float cp = __shfl_sync(gmask, g_cp, t, LANES);
                const float sp = __shfl_sync(gmask, g_sp, t, LANES);
                const float w = __shfl_sync(gmask, g_w, t, LANES);
                // z = e^{i phi}, s = sin(theta). Prefix products over the group's
                // threads of (1 at thread 0, z elsewhere) give z^a at thread a;
                // suffix products of (z below thread used - 1, 1 above) give
                // z^(used - 1 - a), and z^mb = z^(lmax - used + 1) z^(used - 1 - a).
                float pa_re = sub == 0 ? 1.0f : cp, pa_im = sub == 0 ? 0.0f : sp, pa_s = sub == 0 ? 1.0f : st;
                float sf_re = sub < used - 1 ? cp : 1.0f, sf_im = sub < used - 1 ? sp : 0.0f,
                      sf_s = sub < used - 1 ? st : 1.0f;
#pragma unroll
                for (int d = 1; d < LANES; d <<= 1)
                {
                    const float ore = __shfl_up_sync(gmask, pa_re, d, LANES);
                    const float oim = __shfl_up_sync(gmask, pa_im, d, LANES);
                    const float os = __shfl_up_sync(gmask, pa_s, d, LANES);
                    const float dre = __shfl_down_sync(gmask, sf_re, d, LANES);
                    const float dim = __shfl_down_sync(gmask, sf_im, d, LANES);
                    const float ds = __shfl_down_sync(gmask, sf_s, d, LANES);
                    if (sub >= d)
                    {
                        const float nr = pa_re * ore - pa_im * oim;
                        pa_im = pa_re * oim + pa_im * ore;
                        pa_re = nr;
                        pa_s *= os;
                    }
                    if (sub + d < LANES)
                    {
                        const float nr = sf_re * dre - sf_im * dim;
                        sf_im = sf_re * dim + sf_im * dre;
                        sf_re = nr;
                        sf_s *= ds;
                    }
                }
                // z^(used - 1) and s^(used - 1) live at thread used - 1; lmax - used + 1
                // is used - 1 (even lmax) or used (odd lmax)
                float top_re = __shfl_sync(gmask, pa_re, used - 1, LANES);
                float top_im = __shfl_sync(gmask, pa_im, used - 1, LANES);
                float top_s = __shfl_sync(gmask, pa_s, used - 1, LANES);
                if (lmax & 1)
                {
                    const float nr = top_re * cp - top_im * sp;
                    top_im = top_re * sp + top_im * cp;
                    top_re = nr;
                    top_s *= st;
                }
                const float pb_re = top_re * sf_re - top_im * sf_im;
                const float pb_im = top_re * sf_im + top_im * sf_re;
                const float pb_s = top_s * sf_s;
                // normalised Legendre recurrences in l divided by K_m sin^m(theta):
                // R_m = 1, R_{m+1} = sqrt(2m+3) x R_m, R_l = a_lm (x R_{l-1} - b_lm R_{l-2});
                // Q_l^m = K_m sin^m(theta) R_l. Steps 0 .. split-1 run m = ma,
                // the remaining ma steps run m = mb.
                float RA[NL], RB[NL];
#pragma unroll
                for (int kk = 0; kk < NL; ++kk)
                {
                    RA[kk] = lt[kk] == ma ? 1.0f : 0.0f;
                    RB[kk] = lt[kk] == mb ? 1.0f : 0.0f;
                }
                float r_cur = 1.0f, r_prev = 0.0f;
                int m = ma, l = ma;
                float c1 = c1a;
                for (int s = 0; s < lmax; ++s)
                {
                    if (s == split)
                    {
                        m = mb;
                        l = mb;
                        c1 = c1b;
                        r_cur = 1.0f;
                        r_prev = 0.0f;
                    }
                    ++l;
                    const float r = l == m + 1
                        ? c1 * ct * r_cur
                        : s_a[l * (ST_MAX_L + 1) + m] * (ct * r_cur - s_b[l * (ST_MAX_L + 1) + m] * r_prev);
                    r_prev = r_cur;
                    r_cur = r;
                    const bool in_a = s < split;
#pragma unroll
                    for (int kk = 0; kk < NL; ++kk)
                    {
                        if (lt[kk] == l)
                        {
                            if (in_a)
                                RA[kk] = r;
                            else
                                RB[kk] = r;
                        }
                    }
                }
                const float pfa = w * ka * pa_s;
                const float wa_re = pfa * pa_re, wa_im = pfa * pa_im;
                const float pfb = w * kb * pb_s;
                const float wb_re = pfb * pb_re, wb_im = pfb * pb_im;
#pragma unroll
                for (int kk = 0; kk < NL; ++kk)
                {
                    const float ar = RA[kk] * wa_re, ai = RA[kk] * wa_im;
                    accA_re[kk][0] += ar;
                    accA_im[kk][0] += ai;
                    // Y_l^{-m} = (-1)^m conj(Y_l^m)
                    accA_re[kk][1] += sga * ar;
                    accA_im[kk][1] -= sga * ai;
                    const float br = RB[kk] * wb_re, bi = RB[kk] * wb_im;
                    accB_re[kk][0] += br;
                    accB_im[kk][0] += bi;
                    accB_re[kk][1] += sgb * br;
                    accB_im[kk][1] -= sgb * bi;
                }
                tw += w;
            }
        }
        // normalise, write, and reduce ql over the particle's threads (slot kk holds
        // the kk-th smallest l, whose caller index is k)
#pragma unroll
        for (int kk = 0; kk < NL; ++kk)
        {
            if (kk >= ls.nl)
            {
                break;
            }
            const int k = ls.sorted_k[kk];
            const int lk = lt[kk];
            float part = 0.0f;
            float2* row = qlm_out + ls.qlm_offset[k] + static_cast<size_t>(i) * (2 * lk + 1);
            if (has_a && ma <= lk)
            {
                const float qr = accA_re[kk][0] / tw;
                const float qi = accA_im[kk][0] / tw;
                row[ma] = make_float2(qr, qi);
                part += qr * qr + qi * qi;
                if (ma > 0)
                {
                    const float nr = accA_re[kk][1] / tw;
                    const float ni = accA_im[kk][1] / tw;
                    row[lk + ma] = make_float2(nr, ni);
                    part += nr * nr + ni * ni;
                }
            }
            if (has_b && mb <= lk)
            {
                const float qr = accB_re[kk][0] / tw;
                const float qi = accB_im[kk][0] / tw;
                row[mb] = make_float2(qr, qi);
                part += qr * qr + qi * qi;
                const float nr = accB_re[kk][1] / tw;
                const float ni = accB_im[kk][1] / tw;
                row[lk + mb] = make_float2(nr, ni);
                part += nr * nr + ni * ni;
            }
            for (int o = LANES / 2; o > 0; o >>= 1)
            {
                part += __shfl_xor_sync(gmask, part, o, LANES);
            }
            if (sub == 0)
            {
                ql_out[static_cast<size_t>(i) * ls.nl + k] = sqrtf(part * ls.norm[k]);
            }
        }
    }
}

// One l value, bonds spread flat over the lanes: a warp takes per_warp consecutive
// particles (a few bonds each), lane t of a round computes every order m of
// Y_l^m for bond round*32 + t of the warp's particles (one geometry and l(l+1)/2
// recurrence steps per bond, all lanes busy), and a segmented shuffle scan keyed
// by particle adds each particle's part of the round into its shared-memory row.
// Summation order is fixed (tree within a round, rounds in sequence).
template<int L>
__global__ void __launch_bounds__(128)
    k_qlm_flat(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
               const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
               const uint32_t* __restrict__ cnt, const float4* __restrict__ bvd, StLs ls, int weighted,
               uint32_t per_warp, float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    constexpr int NV = 2 * (L + 1) + 1; // re, im for m = 0..L, then the weight (odd: no bank conflicts)
    __shared__ float acc_s[4][32][NV];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    float (*acc)[NV] = acc_s[warp];
    const uint32_t nwarps = gridDim.x * 4;
    for (uint32_t p0 = (blockIdx.x * 4 + warp) * per_warp; p0 < n; p0 += nwarps * per_warp)
    {
        const uint32_t np = min(per_warp, n - p0);
        uint32_t c = 0, sg = 0;
        if (static_cast<uint32_t>(lane) < np)
        {
            c = cnt[p0 + lane];
            sg = seg[p0 + lane];
        }
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(FULL, incl, o);
            if (lane >= o)
                incl += v;
        }
        const uint32_t excl = incl - c;
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        // the warp's bonds are contiguous from the first particle that has any
        const unsigned nz = __ballot_sync(FULL, c > 0);
        const uint32_t base = nz ? __shfl_sync(FULL, sg, __ffs(nz) - 1) : 0u;
#pragma unroll
        for (int v = 0; v < NV; ++v)
            acc[lane][v] = 0.0f;
        __syncwarp();
        for (uint32_t r0 = 0; r0 < total; r0 += 32)
        {
            const uint32_t bb = r0 + static_cast<uint32_t>(lane);
            const bool live = bb < total;
            // particle slot of bond bb: the last slot whose exclusive prefix is <= bb
            int k = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1)
            {
                const uint32_t v = __shfl_sync(FULL, excl, k + step);
                if (v <= bb)
                    k += step;
            }
            float vals[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v)
                vals[v] = 0.0f;
            if (live)
            {
                const uint32_t e = base + bb;
                float dx, dy, dz, d;
                if (bvd != nullptr)
                {
                    const float4 v4 = bvd[e];
                    dx = v4.x;
                    dy = v4.y;
                    dz = v4.z;
                    d = v4.w;
                }
                else
                {
                    const uint32_t i = p0 + static_cast<uint32_t>(k);
                    const uint32_t j = ij[e].y;
                    box_wrap(b, __fsub_rn(pts[3 * (size_t) j], pts[3 * (size_t) i]),
                             __fsub_rn(pts[3 * (size_t) j + 1], pts[3 * (size_t) i + 1]),
                             __fsub_rn(pts[3 * (size_t) j + 2], pts[3 * (size_t) i + 2]), dx, dy, dz);
                    d = dist[e];
                }
                const float w = weighted ? weights[e] : 1.0f;
                float ct, st;
                bond_angle(dz, d, ct, st);
                const float rho = sqrtf(dx * dx + dy * dy);
                float cp = 1.0f, sp = 0.0f;
                if (rho > 0.0f)
                {
                    cp = dx / rho;
                    sp = dy / rho;
                }
                // z^m = e^{i m phi} and s^m by repeated products; Q_L^m = K_m s^m R_L^m
                float zr = 1.0f, zi = 0.0f, sm = 1.0f;
#pragma unroll
                for (int m = 0; m <= L; ++m)
                {
                    if (m > 0)
                    {
                        const float nr = zr * cp - zi * sp;
                        zi = zr * sp + zi * cp;
                        zr = nr;
                        sm *= st;
                    }
                    float r_prev = 0.0f, r_cur = 1.0f;
                    if (L > m)
                    {
                        r_prev = r_cur;
                        r_cur = sqrtf(2.0f * m + 3.0f) * ct * r_prev;
                    }
#pragma unroll
                    for (int l = m + 2; l <= L; ++l)
                    {
                        const float r = c_a[l * (ST_MAX_L + 1) + m] * (ct * r_cur - c_b[l * (ST_MAX_L + 1) + m] * r_prev);
                        r_prev = r_cur;
                        r_cur = r;
                    }
                    const float pf = w * c_K[m] * sm;
                    vals[2 * m] = r_cur * (pf * zr);
                    vals[2 * m + 1] = r_cur * (pf * zi);
                }
                vals[NV - 1] = w;
            }
            // segmented inclusive scan keyed by particle slot (dead lanes get unique keys)
            const int key = live ? k : 32 + lane;
#pragma unroll
            for (int dlt = 1; dlt < 32; dlt <<= 1)
            {
                const int kup = __shfl_up_sync(FULL, key, dlt);
                const bool take = lane >= dlt && kup == key;
#pragma unroll
                for (int v = 0; v < NV; ++v)
                {
                    const float up = __shfl_up_sync(FULL, vals[v], dlt);
                    if (take)
                        vals[v] += up;
                }
            }
            const int knext = __shfl_down_sync(FULL, key, 1);
            if (live && (lane == 31 || knext != key))
            {
#pragma unroll
                for (int v = 0; v < NV; ++v)
                    acc[k][v] += vals[v];
            }
            __syncwarp();
        }
        if (static_cast<uint32_t>(lane) < np)
        {
            const uint32_t i = p0 + lane;
            const float tw = acc[lane][NV - 1];
            float2* row = qlm_out + ls.qlm_offset[0] + static_cast<size_t>(i) * (2 * L + 1);
            float part = 0.0f;
#pragma unroll
            for (int m = 0; m <= L; ++m)
            {
                const float qr = acc[lane][2 * m] / tw;
                const float qi = acc[lane][2 * m + 1] / tw;
                row[m] = make_float2(qr, qi);
                part += qr * qr + qi * qi;
                if (m > 0)
                {
                    // Y_l^{-m} = (-1)^m conj(Y_l^m)
                    const float sgn = (m & 1) ? -1.0f : 1.0f;
                    const float nr = sgn * qr, ni = -sgn * qi;
                    row[L + m] = make_float2(nr, ni);
                    part += nr * nr + ni * ni;
                }
            }
            ql_out[static_cast<size_t>(i) * ls.nl] = sqrtf(part * ls.norm[0]);
        }
        __syncwarp();
    }
}

// One order m per thread (thread m of LANES >= l_max + 1): fewer registers than
// the paired kernel, used when many l values are requested.
template<int LANES, int NL>
__global__ void __launch_bounds__(128)
    k_qlm_m(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
          const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
          const uint32_t* __restrict__ cnt, const float4* __restrict__ bvd, StLs ls, int weighted,
          float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    // recurrence coefficients staged once per block (lanes read different m)
    __shared__ float s_a[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    __shared__ float s_b[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    __shared__ float s_K[ST_MAX_L + 1];
    for (int t = threadIdx.x; t <= ls.max_l * (ST_MAX_L + 1) + ST_MAX_L; t += blockDim.x)
    {
        s_a[t] = c_a[t];
        s_b[t] = c_b[t];
    }
    for (int t = threadIdx.x; t <= ST_MAX_L; t += blockDim.x)
        s_K[t] = c_K[t];
    __syncthreads();

    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES;               // m owned by this thread
    const int group = lane / LANES;             // particle slot within the warp
    const int groups_per_block = blockDim.x / LANES;
    const unsigned gmask = LANES == 32 ? FULL : (((1u << LANES) - 1u) << (group * LANES));
    const int m = sub;
    const float sgn = (m & 1) ? -1.0f : 1.0f;
    // slot kk holds the kk-th smallest requested l
    int lt[NL];
#pragma unroll
    for (int kk = 0; kk < NL; ++kk)
        lt[kk] = kk < ls.nl ? ls.l[ls.sorted_k[kk]] : -1;
    const int lmax = ls.max_l;
    const float km = m <= lmax ? s_K[m] : 0.0f;
    const float c1 = sqrtf(2.0f * m + 3.0f);
    for (uint32_t i = blockIdx.x * groups_per_block + threadIdx.x / LANES; i < n; i += gridDim.x * groups_per_block)
    {
        float acc_re[NL][2];
        float acc_im[NL][2];
#pragma unroll
        for (int k = 0; k < NL; ++k)
        {
            acc_re[k][0] = acc_re[k][1] = acc_im[k][0] = acc_im[k][1] = 0.0f;
        }
        float tw = 0.0f;
        const uint32_t b0 = seg[i];
        const uint32_t nbond = cnt[i];
        float pix = 0.f, piy = 0.f, piz = 0.f;
        if (bvd == nullptr)
        {
            pix = pts[3 * (size_t) i];
            piy = pts[3 * (size_t) i + 1];
            piz = pts[3 * (size_t) i + 2];
        }
        // bonds in batches of LANES: lane t computes the geometry of bond base + t
        // (independent loads in flight), then the group walks the batch with shuffles
        for (uint32_t base = 0; base < nbond; base += LANES)
        {
            float g_ct = 1.0f, g_st = 0.0f, g_cp = 1.0f, g_sp = 0.0f, g_w = 0.0f;
            if (base + sub < nbond)
            {
                const uint32_t e = b0 + base + sub;
                float dx, dy, dz, d;
                if (bvd != nullptr)
                {
                    const float4 v = bvd[e];
                    dx = v.x;
                    dy = v.y;
                    dz = v.z;
                    d = v.w;
                }
                else
                {
                    const uint32_t j = ij[e].y;
                    box_wrap(b, __fsub_rn(pts[3 * (size_t) j], pix), __fsub_rn(pts[3 * (size_t) j + 1], piy),
                             __fsub_rn(pts[3 * (size_t) j + 2], piz), dx, dy, dz);
                    d = dist[e];
                }
                g_w = weighted ? weights[e] : 1.0f;
                bond_angle(dz, d, g_ct, g_st);
                const float rho = sqrtf(dx * dx + dy * dy);
                if (rho > 0.0f)
                {
                    g_cp = dx / rho;
                    g_sp = dy / rho;
                }
            }
            const uint32_t nb_here = min(static_cast<uint32_t>(LANES), nbond - base);
            for (uint32_t t = 0; t < nb_here; ++t)
            {
                const float ct = __shfl_sync(gmask, g_ct, t, LANES);
                const float st = __shfl_sync(gmask, g_st, t, LANES);
                const float cp = __shfl_sync(gmask, g_cp, t, LANES);
                const float sp = __shfl_sync(gmask, g_sp, t, LANES);
                const float w = __shfl_sync(gmask, g_w, t, LANES);
                // e^{i m phi} and sin^m(theta) for every lane at once: an inclusive
                // prefix product over the group's lanes of (1 at lane 0, z elsewhere)
                // leaves z^m at lane m in log2(LANES) uniform steps.
                float em_re = sub == 0 ? 1.0f : cp, em_im = sub == 0 ? 0.0f : sp, sm = sub == 0 ? 1.0f : st;
#pragma unroll
                for (int d = 1; d < LANES; d <<= 1)
                {
                    const float ore = __shfl_up_sync(gmask, em_re, d, LANES);
                    const float oim = __shfl_up_sync(gmask, em_im, d, LANES);
                    const float os = __shfl_up_sync(gmask, sm, d, LANES);
                    if (sub >= d)
                    {
                        const float nr = em_re * ore - em_im * oim;
                        em_im = em_re * oim + em_im * ore;
                        em_re = nr;
                        sm *= os;
                    }
                }
                // normalised Legendre recurrence in l for this lane's m, divided by
                // K_m sin^m(theta): R_m = 1, R_{m+1} = sqrt(2m+3) x R_m,
                // R_l = a_lm (x R_{l-1} - b_lm R_{l-2}); Q_l^m = K_m sin^m(theta) R_l
                float r_cur = 1.0f, r_prev = 0.0f;
                float R[NL];
#pragma unroll
                for (int kk = 0; kk < NL; ++kk)
                    R[kk] = lt[kk] == m ? 1.0f : 0.0f;
                for (int l = m + 1; l <= lmax; ++l)
                {
                    const float r = l == m + 1
                        ? c1 * ct * r_cur
                        : s_a[l * (ST_MAX_L + 1) + m] * (ct * r_cur - s_b[l * (ST_MAX_L + 1) + m] * r_prev);
                    r_prev = r_cur;
                    r_cur = r;
#pragma unroll
                    for (int kk = 0; kk < NL; ++kk)
                    {
                        if (lt[kk] == l)
                            R[kk] = r;
                    }
                }
                const float pf = w * km * sm;
                const float wre = pf * em_re;
                const float wim = pf * em_im;
#pragma unroll
                for (int kk = 0; kk < NL; ++kk)
                {
                    const float yr = R[kk] * wre;
                    const float yi = R[kk] * wim;
                    acc_re[kk][0] += yr;
                    acc_im[kk][0] += yi;
                    // Y_l^{-m} = (-1)^m conj(Y_l^m)
                    acc_re[kk][1] += sgn * yr;
                    acc_im[kk][1] -= sgn * yi;
                }
                tw += w;
            }
        }
        // normalise, write, and reduce ql over the particle's lanes (slot kk holds
        // the kk-th smallest l, whose caller index is k)
#pragma unroll
        for (int kk = 0; kk < NL; ++kk)
        {
            if (kk >= ls.nl)
            {
                break;
            }
            const int k = ls.sorted_k[kk];
            const int lk = lt[kk];
            float part = 0.0f;
            if (m <= lk)
            {
                const float qr = acc_re[kk][0] / tw;
                const float qi = acc_im[kk][0] / tw;
                float2* row = qlm_out + ls.qlm_offset[k] + static_cast<size_t>(i) * (2 * lk + 1);
                row[m] = make_float2(qr, qi);
                part = qr * qr + qi * qi;
                if (m > 0)
                {
                    const float nr = acc_re[kk][1] / tw;
                    const float ni = acc_im[kk][1] / tw;
                    row[lk + m] = make_float2(nr, ni);
                    part += nr * nr + ni * ni;
                }
            }
            for (int o = LANES / 2; o > 0; o >>= 1)
            {
                part += __shfl_xor_sync(gmask, part, o, LANES);
            }
            if (sub == 0)
            {
                ql_out[static_cast<size_t>(i) * ls.nl + k] = sqrtf(part * ls.norm[k]);
            }
        }
    }
}

// Neighbour averaging: ave(i) = (sum_j qlm(j) + qlm(i)) / (1 + n_i). Per l, the
// neighbour indices of LANES bonds are loaded at once (one per lane) and
// broadcast, so the row gathers do not wait on the index loads one by one.
template<int LANES>
__global__ void __launch_bounds__(128)
    k_ave(uint32_t n, const uint2* __restrict__ ij, const uint32_t* __restrict__ bj, const uint32_t* __restrict__ seg,
          const uint32_t* __restrict__ cnt, StLs ls, const float2* __restrict__ qlm, float2* __restrict__ ave,
          float* __restrict__ ql_ave, const uint32_t* __restrict__ order)
{
    const int lane = threadIdx.x & 31;
    const int sub = lane % LANES;
    const int group = lane / LANES;
    const int groups_per_block = blockDim.x / LANES;
    const unsigned gmask = LANES == 32 ? FULL : (((1u << LANES) - 1u) << (group * LANES));
    const int m = sub;
    for (uint32_t t = blockIdx.x * groups_per_block + threadIdx.x / LANES; t < n; t += gridDim.x * groups_per_block)
    {
        // particles in the given order (cell order: neighbours share qlm rows in L2), else by index
        const uint32_t i = order != nullptr ? order[t] : t;
        const uint32_t b0 = seg[i];
        const uint32_t nbond = cnt[i];
        const float cntf = static_cast<float>(1u + nbond);
        for (int k = 0; k < ls.nl; ++k)
        {
            const int l = ls.l[k];
            const float2* base_k = qlm + ls.qlm_offset[k];
            float pr = 0.f, pim = 0.f, nr = 0.f, nim = 0.f;
            for (uint32_t base = 0; base < nbond; base += LANES)
            {
                const uint32_t jl = base + sub < nbond ? (bj != nullptr ? bj[b0 + base + sub] : ij[b0 + base + sub].y) : 0u;
                const uint32_t nb_here = min(static_cast<uint32_t>(LANES), nbond - base);
                for (uint32_t t = 0; t < nb_here; ++t)
                {
                    const uint32_t j = __shfl_sync(gmask, jl, t, LANES);
                    if (m <= l)
                    {
                        const float2* rj = base_k + static_cast<size_t>(j) * (2 * l + 1);
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
                }
            }
            float part = 0.0f;
            if (m <= l)
            {
                const float2* ri = base_k + static_cast<size_t>(i) * (2 * l + 1);
                const float2 a = ri[m];
                const float qr = (pr + a.x) / cntf;
                const float qi = (pim + a.y) / cntf;
                float2* out = ave + ls.qlm_offset[k] + static_cast<size_t>(i) * (2 * l + 1);
                out[m] = make_float2(qr, qi);
                part = qr * qr + qi * qi;
                if (m > 0)
                {
                    const float2 c = ri[l + m];
                    const float vr = (nr + c.x) / cntf;
                    const float vi = (nim + c.y) / cntf;
                    out[l + m] = make_float2(vr, vi);
                    part += vr * vr + vi * vi;
                }
            }
            for (int o = LANES / 2; o > 0; o >>= 1)
            {
                part += __shfl_xor_sync(gmask, part, o, LANES);
            }
            if (sub == 0)
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
    // the block's rows (coalesced), then the l's Wigner-3j coefficients (every
    // thread reads coefficient c at the same time: a shared-memory broadcast)
    float* w3s = reinterpret_cast<float*>(rows + blockDim.x * static_cast<uint32_t>(nm));
    for (uint32_t e = threadIdx.x; e < blockDim.x * static_cast<uint32_t>(nm); e += blockDim.x)
    {
        const uint32_t gi = i0 + e / nm;
        rows[e] = gi < n ? src[qlm_offset + static_cast<size_t>(i0) * nm + e] : make_float2(0.f, 0.f);
    }
    const int nterms = 3 * l * l + 3 * l + 1;
    for (int e = threadIdx.x; e < nterms; e += blockDim.x)
        w3s[e] = w3j[e];
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
            const float term = w3s[c] * (abr * cq.x - abi * cq.y);
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

// Threads per particle of k_qlm: one per pair of orders (m, l_max - m).
static int pair_lanes_for(int max_l)
{
    const int used = max_l / 2 + 1;
    return used <= 4 ? 4 : (used <= 8 ? 8 : 16);
}

namespace {
template<int L>
void qlm_flat(const DevBox& box, const float* pts, uint32_t n, const uint2* ij, const float* dist, const float* weights,
              const uint32_t* seg, const uint32_t* cnt, const StLs& ls, int weighted, float2* qlm, float* ql,
              cudaStream_t s, const float4* bond_vd, uint32_t per_warp)
{
    const uint32_t per_block = 4 * per_warp;
    uint32_t blocks = (n + per_block - 1) / per_block;
    const uint32_t cap = static_cast<uint32_t>(sm_count()) * 16;
    blocks = blocks < cap ? blocks : cap;
    ProfScope prof_("k_qlm_flat", s);
    k_qlm_flat<L><<<blocks, 128, 0, s>>>(box, pts, n, ij, dist, weights, seg, cnt, bond_vd, ls, weighted, per_warp,
                                         qlm, ql);
}
} // namespace

void launch_qlm(const DevBox& box, const float* pts, uint32_t n, const uint2* ij, const float* dist,
                const float* weights, const uint32_t* seg, const uint32_t* cnt, const StLs& ls, int weighted,
                float2* qlm, float* ql, cudaStream_t s, const float4* bond_vd, double mean_bonds)
{
    if (n == 0)
    {
        return;
    }
    if (ls.nl == 1 && ls.max_l <= 12)
    {
        // one l: bonds flat over the lanes, about three rounds of 32 per warp
        const double mb = mean_bonds > 0.0 ? mean_bonds : 24.0;
        const uint32_t per_warp = static_cast<uint32_t>(std::min(32.0, std::max(1.0, std::floor(96.0 / mb))));
        switch (ls.max_l)
        {
        case 0: qlm_flat<0>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 1: qlm_flat<1>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 2: qlm_flat<2>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 3: qlm_flat<3>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 4: qlm_flat<4>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 5: qlm_flat<5>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 6: qlm_flat<6>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 7: qlm_flat<7>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 8: qlm_flat<8>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 9: qlm_flat<9>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 10: qlm_flat<10>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        case 11: qlm_flat<11>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        default: qlm_flat<12>(box, pts, n, ij, dist, weights, seg, cnt, ls, weighted, qlm, ql, s, bond_vd, per_warp); return;
        }
    }
    const int nlt = ls.nl <= 1 ? 1 : (ls.nl <= 2 ? 2 : (ls.nl <= 5 ? 5 : ST_MAX_NL));
    // paired orders for one or two l values; with more, the doubled accumulators
    // cost more registers than the divergence they remove
    const bool paired = nlt <= 2;
    const int lanes = paired ? pair_lanes_for(ls.max_l) : lanes_for(ls.max_l);
    const uint32_t groups = 128 / lanes;
    uint32_t blocks = (n + groups - 1) / groups;
    const uint32_t cap = static_cast<uint32_t>(sm_count()) * 16;
    blocks = blocks < cap ? blocks : cap;
    auto go = [&](auto kernel, const char* name) {
        ProfScope prof_(name, s);
        kernel<<<blocks, 128, 0, s>>>(box, pts, n, ij, dist, weights, seg, cnt, bond_vd, ls, weighted, qlm, ql);
    };
    if (!paired)
    {
        if (lanes == 8)
            go(nlt == 5 ? k_qlm_m<8, 5> : k_qlm_m<8, ST_MAX_NL>, "k_qlm_m<8>");
        else if (lanes == 16)
            go(nlt == 5 ? k_qlm_m<16, 5> : k_qlm_m<16, ST_MAX_NL>, "k_qlm_m<16>");
        else
            go(nlt == 5 ? k_qlm_m<32, 5> : k_qlm_m<32, ST_MAX_NL>, "k_qlm_m<32>");
    }
    else if (lanes == 4)
    {
        if (nlt == 1)
            go(k_qlm<4, 1>, "k_qlm<4>");
        else
            go(k_qlm<4, 2>, "k_qlm<4>");
    }
    else if (lanes == 8)
    {
        if (nlt == 1)
            go(k_qlm<8, 1>, "k_qlm<8>");
        else
            go(k_qlm<8, 2>, "k_qlm<8>");
    }
    else
    {
        if (nlt == 1)
            go(k_qlm<16, 1>, "k_qlm<16>");
        else
            go(k_qlm<16, 2>, "k_qlm<16>");
    }
}

void launch_ave(uint32_t n, const uint2* ij, const uint32_t* seg, const uint32_t* cnt, const StLs& ls,
                const float2* qlm, float2* ave, float* ql_ave, cudaStream_t s, const uint32_t* bond_j,
                const uint32_t* order)
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
            k_ave<8><<<blocks, 128, 0, s>>>(n, ij, bond_j, seg, cnt, ls, qlm, ave, ql_ave, order);
        }
    else if (lanes == 16)
        {
            ProfScope prof_("k_ave<16>", s);
            k_ave<16><<<blocks, 128, 0, s>>>(n, ij, bond_j, seg, cnt, ls, qlm, ave, ql_ave, order);
        }
    else
        {
            ProfScope prof_("k_ave<32>", s);
            k_ave<32><<<blocks, 128, 0, s>>>(n, ij, bond_j, seg, cnt, ls, qlm, ave, ql_ave, order);
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
    const size_t smem = 128 * static_cast<size_t>(2 * l + 1) * sizeof(float2) +
                        static_cast<size_t>(3 * l * l + 3 * l + 1) * sizeof(float);
    static bool configured = false;
    if (!configured)
    {
        cudaFuncSetAttribute(k_wl, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(128 * (2 * ST_MAX_L + 1) * sizeof(float2) +
                                              (3 * ST_MAX_L * ST_MAX_L + 3 * ST_MAX_L + 1) * sizeof(float)));
        configured = true;
    }
    {
        ProfScope prof_("k_wl", s);
        k_wl<<<(n + 127) / 128, 128, smem, s>>>(n, l, k, ls.nl, ls.qlm_offset[k], src, w3j_dev, qnorm, normalize,
                                                ls.norm[k], wl);
    }
}


} // namespace fg
