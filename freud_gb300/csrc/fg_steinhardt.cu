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
// k_wl: thread per particle, the Wigner-3j triple sums over classes of equal terms in float-float.
// The FP64 system sums (qlm or averaged qlm over the particles, divided by N)
// are taken by the per-frame column-sum kernels of fg_batch.cu.
#include <algorithm>
#include <array>
#include <cstring>
#include <utility>
#include <vector>
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
// float-float copies (hi, lo) of K_m and of the recurrence coefficients, with
// a_{m+1,m} = sqrt(2m + 3) and b_{m+1,m} = 0 so one formula covers every step
__constant__ float2 c_Kff[ST_MAX_L + 1];
__constant__ float2 c_aff[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
__constant__ float2 c_bff[(ST_MAX_L + 1) * (ST_MAX_L + 1)];

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
// recurrence steps per bond, all lanes busy) and stores them in a shared-memory
// row; then lanes take (particle, value) pairs, each adding its particle's bonds
// of the round for one value in bond order, into the particle's accumulator
// (values of up to two particles at a time when a row has at most 16 values).
// Summation order is fixed (bond order within a round, rounds in sequence).
template<int L>
__global__ void __launch_bounds__(128)
    k_qlm_flat(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
               const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
               const uint32_t* __restrict__ cnt, const float4* __restrict__ bvd, StLs ls, int weighted,
               uint32_t per_warp, float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    constexpr int NV = 2 * (L + 1) + 1; // re, im for m = 0..L, then the weight (odd: no bank conflicts)
    constexpr int SEGS = NV <= 16 ? 2 : 1; // particles summed at a time
    constexpr int SPAN = 32 / SEGS;        // lanes per particle (value v = lane % SPAN)
    static_assert(NV <= 32, "a row's values must fit the lanes of a warp");
    __shared__ float acc_s[4][32][NV];
    __shared__ float val_s[4][32][NV];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    float (*acc)[NV] = acc_s[warp];
    float (*val)[NV] = val_s[warp];
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
            // bond bb is bond bb - excl of its particle's segment (segments need not be
            // contiguous from one particle to the next)
            const uint32_t e = __shfl_sync(FULL, sg, k) + (bb - __shfl_sync(FULL, excl, k));
            float vals[NV];
#pragma unroll
            for (int v = 0; v < NV; ++v)
                vals[v] = 0.0f;
            if (live)
            {
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
            if (live)
            {
#pragma unroll
                for (int v = 0; v < NV; ++v)
                    val[lane][v] = vals[v];
            }
            __syncwarp();
            // the round's bonds are lanes [0, nlive), particle slots kf .. kl (bonds of
            // one slot are consecutive lanes; slots between with no bonds add nothing)
            const int nlive = static_cast<int>(min(32u, total - r0));
            const int kf = __shfl_sync(FULL, k, 0);
            const int kl = __shfl_sync(FULL, k, nlive - 1);
            const int v = lane % SPAN;
            for (int s0 = kf; s0 <= kl; s0 += SEGS)
            {
                const int sl = s0 + lane / SPAN;
                const int src = sl < 32 ? sl : 31;
                const int xs = static_cast<int>(__shfl_sync(FULL, excl, src)) - static_cast<int>(r0);
                const int xe = xs + static_cast<int>(__shfl_sync(FULL, c, src));
                if (sl <= kl && v < NV)
                {
                    const int lo = xs > 0 ? xs : 0;
                    const int hi = xe < nlive ? xe : nlive;
                    if (hi > lo)
                    {
                        float sum = val[lo][v];
                        for (int t = lo + 1; t < hi; ++t)
                            sum += val[t][v];
                        acc[sl][v] += sum;
                    }
                }
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

// Float-float arithmetic: a value is the unevaluated sum h + l of two floats.
// Products by Dekker's method with the exact FMA remainder; sums by Knuth's
// TwoSum followed by a Fast2Sum renormalisation (the "sloppy" double-float add
// of Hida, Li and Bailey's QD library). Each operation keeps about 2^-44 of the
// value, so a 31-step Legendre recurrence stays far below one float ulp. Every
// operation is an explicit round-to-nearest intrinsic, which the compiler neither
// contracts nor reorders.
struct ffl
{
    float h, l;
};

__device__ __forceinline__ ffl ff_mul(ffl a, ffl b)
{
    const float p = __fmul_rn(a.h, b.h);
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return {p, e};
}

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ ffl ff_add(ffl a, ffl b)
{
    float s, e;
    two_sum(a.h, b.h, s, e);
    e = __fadd_rn(e, __fadd_rn(a.l, b.l));
    const float h = __fadd_rn(s, e);
    return {h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ ffl ff_sub(ffl a, ffl b)
{
    return ff_add(a, {-b.h, -b.l});
}

// TwoSum without the renormalisation: the pair (s, e) may carry |e| above half an
// ulp of s after a cancellation, which keeps its value to about 2^-47 of the
// operands' magnitude, as later products and sums need
__device__ __forceinline__ ffl ff_add_lazy(ffl a, ffl b)
{
    float s, e;
    two_sum(a.h, b.h, s, e);
    return {s, __fadd_rn(e, __fadd_rn(a.l, b.l))};
}

__device__ __forceinline__ ffl ff_sub_lazy(ffl a, ffl b)
{
    return ff_add_lazy(a, {-b.h, -b.l});
}

__device__ __forceinline__ ffl ff_sqrt(ffl v)
{
    if (!(v.h > 0.0f))
        return {0.0f, 0.0f};
    const float s = __fsqrt_rn(v.h);
    const float r = __fadd_rn(__fmaf_rn(-s, s, v.h), v.l);
    return {s, __fdiv_rn(r, __fmul_rn(2.0f, s))};
}

// acc += y, hi parts by TwoSum, the rounding errors and lo parts summed apart
__device__ __forceinline__ void ff_acc(float& ah, float& al, ffl y)
{
    float s, e;
    two_sum(ah, y.h, s, e);
    ah = s;
    al = __fadd_rn(al, __fadd_rn(e, y.l));
}

// (h + l) / w rounded to float: quotient, exact remainder, one correction
__device__ __forceinline__ float ff_div_f(float h, float l, float w)
{
    const float q = __fdiv_rn(h, w);
    const float r = __fadd_rn(__fmaf_rn(-q, w, h), l);
    return __fadd_rn(q, __fdiv_rn(r, w));
}

// Geometry of one bond in float-float, as the FP64 oracle takes it:
// cos(theta) = clamp(dz / d) (Steinhardt.cc:163-172), sin(theta) =
// sqrt(1 - cos^2), and w = sin(theta) e^{i phi} with e^{i phi} = (dx + i dy) / rho,
// phi = atan2(dy, dx) (Steinhardt.cc:160).
struct BondFF
{
    ffl ct;     // cos(theta)
    ffl wr, wi; // sin(theta) e^{i phi}
    float w;    // bond weight (0 for an empty slot)
};

__device__ __forceinline__ BondFF bond_ff(float dx, float dy, float dz, float d, float w)
{
    BondFF g;
    g.w = w;
    g.ct = {1.0f, 0.0f};
    g.wr = {0.0f, 0.0f};
    g.wi = {0.0f, 0.0f};
    if (d == 0.0f)
        return g;
    const float hi = __fdiv_rn(dz, d);
    const float lo = __fdiv_rn(__fmaf_rn(-hi, d, dz), d);
    if (hi > 1.0f || (hi == 1.0f && lo >= 0.0f))
        return g;
    if (hi < -1.0f || (hi == -1.0f && lo <= 0.0f))
    {
        g.ct = {-1.0f, 0.0f};
        return g;
    }
    g.ct = {hi, lo};
    const ffl c2 = ff_mul(g.ct, g.ct);
    const ffl st = ff_sqrt(ff_sub({1.0f, 0.0f}, c2));
    // rho^2 = dx^2 + dy^2 exactly as two float-float products summed
    const float px = __fmul_rn(dx, dx), py = __fmul_rn(dy, dy);
    const ffl r2 = ff_add({px, __fmaf_rn(dx, dx, -px)}, {py, __fmaf_rn(dy, dy, -py)});
    if (!(r2.h > 0.0f))
    {
        // on the z axis: atan2(+-0, x) is 0 for x = +0 and pi for x = -0
        g.wr = {signbit(dx) ? -st.h : st.h, signbit(dx) ? -st.l : st.l};
        return g;
    }
    const ffl rho = ff_sqrt(r2);
    const float q = __frcp_rn(rho.h);
    float e = __fmaf_rn(-rho.h, q, 1.0f);
    e = __fmaf_rn(-rho.l, q, e);
    const ffl inv = {q, __fmul_rn(e, q)};
    const ffl sinv = ff_mul(st, inv);
    g.wr = ff_mul(sinv, {dx, 0.0f});
    g.wi = ff_mul(sinv, {dy, 0.0f});
    return g;
}

// Every Y_l^m of a bond in float-float (Wl path): thread per particle, BP bonds
// per pass (their recurrences share the coefficient loads and give each step BP
// independent chains). Per order m the power (w sin(theta) e^{i phi})^m is one
// complex float-float product from the previous order's, the prefactor K_m times
// it, then the normalised recurrence R_{l+1} = a (ct R_l - b R_{l-1}) from R_m = 1
// up to l_max, and at each requested l the term R_l x prefactor is added to the
// particle's float-float sum of (l, m) in shared memory (acc[slot][thread]:
// re hi, re lo, im hi, im lo). The weights are real, so the negative orders are
// (-1)^m conj of the sums. The final division by the total weight rounds once,
// so each qlm is the FP64 value to within about one float ulp. Rows are written
// through the warp's shared-memory sums, one particle's row per pass, coalesced.
template<int T, int BP>
__global__ void __launch_bounds__(T, 256 / T)
    k_qlm_ff(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
             const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
             const uint32_t* __restrict__ cnt, const float4* __restrict__ bvd, StLs ls, int weighted,
             float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    extern __shared__ float4 acc[]; // [slots][T]
    __shared__ int s_lt[ST_MAX_NL + 1];
    __shared__ int s_base[ST_MAX_NL + 1];
    __shared__ int s_k[ST_MAX_NL];
    __shared__ size_t s_off[ST_MAX_NL];
    __shared__ float s_norm[ST_MAX_NL];
    __shared__ int s_slot0[ST_MAX_L + 2]; // slot of (l, 0) for a requested l
    if (threadIdx.x == 0)
    {
        int o = 0;
        for (int kk = 0; kk < ls.nl; ++kk)
        {
            const int k = ls.sorted_k[kk];
            s_k[kk] = k;
            s_lt[kk] = ls.l[k];
            s_base[kk] = o;
            s_off[kk] = ls.qlm_offset[k];
            s_norm[kk] = ls.norm[k];
            s_slot0[ls.l[k]] = o;
            o += ls.l[k] + 1;
        }
        s_lt[ls.nl] = -1;
        s_base[ls.nl] = o;
    }
    __syncthreads();
    const int nl = ls.nl;
    const int lmax = ls.max_l;
    const int nslot = s_base[nl];
    unsigned req = 0; // bit l: l requested
    for (int kk = 0; kk < nl; ++kk)
        req |= 1u << s_lt[kk];
    const int lane = threadIdx.x & 31;
    float4* my = acc + threadIdx.x;
    for (uint32_t i0 = blockIdx.x * T; i0 < n; i0 += gridDim.x * T)
    {
        const uint32_t i = i0 + threadIdx.x;
        for (int o = 0; o < nslot; ++o)
            my[o * T] = make_float4(0.f, 0.f, 0.f, 0.f);
        float tw = 0.0f;
        if (i < n)
        {
            const uint32_t b0 = seg[i];
            const uint32_t nbond = cnt[i];
            float pix = 0.f, piy = 0.f, piz = 0.f;
            if (bvd == nullptr)
            {
                pix = pts[3 * (size_t) i];
                piy = pts[3 * (size_t) i + 1];
                piz = pts[3 * (size_t) i + 2];
            }
            for (uint32_t e0 = 0; e0 < nbond; e0 += BP)
            {
                BondFF g[BP];
#pragma unroll
                for (int u = 0; u < BP; ++u)
                {
                    float dx = 0.f, dy = 0.f, dz = 0.f, d = 0.f, w = 0.f;
                    if (e0 + u < nbond)
                    {
                        const uint32_t e = b0 + e0 + u;
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
                        w = weighted ? weights[e] : 1.0f;
                    }
                    g[u] = bond_ff(dx, dy, dz, d, w);
                    tw = __fadd_rn(tw, w);
                }
                // weight x (sin(theta) e^{i phi})^m, starting at m = 0
                ffl pr[BP], pi[BP];
#pragma unroll
                for (int u = 0; u < BP; ++u)
                {
                    pr[u] = {g[u].w, 0.0f};
                    pi[u] = {0.0f, 0.0f};
                }
                for (int m = 0; m <= lmax; ++m)
                {
                    if (m > 0)
                    {
#pragma unroll
                        for (int u = 0; u < BP; ++u)
                        {
                            const ffl nr = ff_sub_lazy(ff_mul(pr[u], g[u].wr), ff_mul(pi[u], g[u].wi));
                            pi[u] = ff_add_lazy(ff_mul(pr[u], g[u].wi), ff_mul(pi[u], g[u].wr));
                            pr[u] = nr;
                        }
                    }
                    const float2 kf = c_Kff[m];
                    const ffl K = {kf.x, kf.y};
                    ffl fr[BP], fi[BP], r1[BP], r0[BP];
#pragma unroll
                    for (int u = 0; u < BP; ++u)
                    {
                        fr[u] = ff_mul(K, pr[u]);
                        fi[u] = ff_mul(K, pi[u]);
                        r1[u] = {1.0f, 0.0f};
                        r0[u] = {0.0f, 0.0f};
                    }
                    for (int l = m;; ++l)
                    {
                        if ((req >> l) & 1u)
                        {
                            float4* slot = my + (s_slot0[l] + m) * T;
                            float4 v = *slot;
#pragma unroll
                            for (int u = 0; u < BP; ++u)
                            {
                                ff_acc(v.x, v.y, ff_mul(r1[u], fr[u]));
                                ff_acc(v.z, v.w, ff_mul(r1[u], fi[u]));
                            }
                            *slot = v;
                        }
                        if (l == lmax)
                            break;
                        const float2 af = c_aff[(l + 1) * (ST_MAX_L + 1) + m];
                        const float2 bf = c_bff[(l + 1) * (ST_MAX_L + 1) + m];
#pragma unroll
                        for (int u = 0; u < BP; ++u)
                        {
                            const ffl t = ff_sub_lazy(ff_mul(g[u].ct, r1[u]), ff_mul({bf.x, bf.y}, r0[u]));
                            r0[u] = r1[u];
                            r1[u] = ff_mul({af.x, af.y}, t);
                        }
                    }
                }
            }
        }
        // sums -> qlm (m >= 0) in place, and ql
        if (i < n)
        {
            for (int kk = 0; kk < nl; ++kk)
            {
                const int l = s_lt[kk];
                float part = 0.0f;
                for (int m = 0; m <= l; ++m)
                {
                    float4* slot = my + (s_base[kk] + m) * T;
                    const float4 v = *slot;
                    const float qr = ff_div_f(v.x, v.y, tw);
                    const float qi = ff_div_f(v.z, v.w, tw);
                    slot->x = qr;
                    slot->y = qi;
                    const float sq = __fmaf_rn(qr, qr, __fmul_rn(qi, qi));
                    part = __fadd_rn(part, m > 0 ? __fmul_rn(2.0f, sq) : sq);
                }
                ql_out[static_cast<size_t>(i) * nl + s_k[kk]] = sqrtf(part * s_norm[kk]);
            }
        }
        __syncwarp();
        // the warp's rows: (2l + 1) consecutive float2 per particle, particles consecutive
        const uint32_t w0 = i0 + (threadIdx.x & ~31u);
        const int wcol = threadIdx.x & ~31;
        for (int kk = 0; kk < nl; ++kk)
        {
            const int l = s_lt[kk];
            const int width = 2 * l + 1;
            float2* out = qlm_out + s_off[kk] + static_cast<size_t>(w0) * width;
            for (int p = 0; p < 32 && w0 + p < n; ++p)
            {
                for (int c = lane; c < width; c += 32)
                {
                    const int m = c <= l ? c : c - l;
                    const float4 v = acc[(s_base[kk] + m) * T + wcol + p];
                    float2 q = make_float2(v.x, v.y);
                    if (c > l)
                        q = (m & 1) ? make_float2(-v.x, v.y) : make_float2(v.x, -v.y);
                    out[static_cast<size_t>(p) * width + c] = q;
                }
            }
        }
        __syncwarp();
    }
}

// The float-float harmonics with two threads per particle: thread parity p takes
// the orders m = p, p + 2, ... (powers stepped by (sin(theta) e^{i phi})^2), so a
// particle's float-float sums (one slot per requested (l, m) with m of the
// thread's parity) take half the shared memory per thread and twice the particles
// fit an SM. Both threads of a pair run the l loop of the pair's even order 2u:
// the odd thread (m = 2u + 1) takes the step l = 2u with R = 0 and starts at
// R_m = 1, so the two see every requested l in the same iteration. Sums, their
// order and the rounding are those of k_qlm_ff.
template<int T, int BP>
__global__ void __launch_bounds__(T, 512 / T)
    k_qlm_ff2(DevBox b, const float* __restrict__ pts, uint32_t n, const uint2* __restrict__ ij,
              const float* __restrict__ dist, const float* __restrict__ weights, const uint32_t* __restrict__ seg,
              const uint32_t* __restrict__ cnt, const float4* __restrict__ bvd, StLs ls, int weighted,
              float2* __restrict__ qlm_out, float* __restrict__ ql_out)
{
    extern __shared__ float4 acc[]; // [slots of one parity][T]
    __shared__ int s_lt[ST_MAX_NL + 1];
    __shared__ int s_k[ST_MAX_NL];
    __shared__ size_t s_off[ST_MAX_NL];
    __shared__ float s_norm[ST_MAX_NL];
    __shared__ int s_pb[2][ST_MAX_L + 2]; // slot of (l, m = parity) for a requested l, per parity
    __shared__ int s_np;                  // slots of the larger parity
    if (threadIdx.x == 0)
    {
        int o0 = 0, o1 = 0;
        for (int kk = 0; kk < ls.nl; ++kk)
        {
            const int k = ls.sorted_k[kk];
            const int l = ls.l[k];
            s_k[kk] = k;
            s_lt[kk] = l;
            s_off[kk] = ls.qlm_offset[k];
            s_norm[kk] = ls.norm[k];
            s_pb[0][l] = o0;
            s_pb[1][l] = o1;
            o0 += l / 2 + 1;
            o1 += (l + 1) / 2;
        }
        s_lt[ls.nl] = -1;
        s_np = o0 > o1 ? o0 : o1;
    }
    __syncthreads();
    const int nl = ls.nl;
    const int lmax = ls.max_l;
    const int par = threadIdx.x & 1;
    const int lane = threadIdx.x & 31;
    unsigned req = 0;
    for (int kk = 0; kk < nl; ++kk)
        req |= 1u << s_lt[kk];
    const int* pb = s_pb[par];
    float4* my = acc + threadIdx.x;
    const int np = s_np;
    constexpr int PPB = T / 2; // particles per block
    for (uint32_t i0 = blockIdx.x * PPB; i0 < n; i0 += gridDim.x * PPB)
    {
        const uint32_t i = i0 + (threadIdx.x >> 1);
        for (int o = 0; o < np; ++o)
            my[o * T] = make_float4(0.f, 0.f, 0.f, 0.f);
        float tw = 0.0f;
        if (i < n)
        {
            const uint32_t b0 = seg[i];
            const uint32_t nbond = cnt[i];
            float pix = 0.f, piy = 0.f, piz = 0.f;
            if (bvd == nullptr)
            {
                pix = pts[3 * (size_t) i];
                piy = pts[3 * (size_t) i + 1];
                piz = pts[3 * (size_t) i + 2];
            }
            for (uint32_t e0 = 0; e0 < nbond; e0 += BP)
            {
                BondFF g[BP];
                ffl w2r[BP], w2i[BP];
                ffl pr[BP], pi[BP];
#pragma unroll
                for (int u = 0; u < BP; ++u)
                {
                    float dx = 0.f, dy = 0.f, dz = 0.f, d = 0.f, w = 0.f;
                    if (e0 + u < nbond)
                    {
                        const uint32_t e = b0 + e0 + u;
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
                        w = weighted ? weights[e] : 1.0f;
                    }
                    g[u] = bond_ff(dx, dy, dz, d, w);
                    tw = __fadd_rn(tw, w);
                    // (s e^{i phi})^2, and the power of order par times the weight
                    w2r[u] = ff_sub_lazy(ff_mul(g[u].wr, g[u].wr), ff_mul(g[u].wi, g[u].wi));
                    w2i[u] = ff_add_lazy(ff_mul(g[u].wr, g[u].wi), ff_mul(g[u].wi, g[u].wr));
                    if (par)
                    {
                        pr[u] = ff_mul(g[u].wr, {g[u].w, 0.0f});
                        pi[u] = ff_mul(g[u].wi, {g[u].w, 0.0f});
                    }
                    else
                    {
                        pr[u] = {g[u].w, 0.0f};
                        pi[u] = {0.0f, 0.0f};
                    }
                }
                for (int m0 = 0; m0 <= lmax; m0 += 2)
                {
                    const int m = m0 + par; // may exceed lmax for the odd thread
                    if (m0 > 0)
                    {
#pragma unroll
                        for (int u = 0; u < BP; ++u)
                        {
                            const ffl nr = ff_sub_lazy(ff_mul(pr[u], w2r[u]), ff_mul(pi[u], w2i[u]));
                            pi[u] = ff_add_lazy(ff_mul(pr[u], w2i[u]), ff_mul(pi[u], w2r[u]));
                            pr[u] = nr;
                        }
                    }
                    const float2 kf = c_Kff[m <= ST_MAX_L ? m : ST_MAX_L];
                    const ffl K = {kf.x, kf.y};
                    ffl fr[BP], fi[BP], r1[BP], r0[BP];
#pragma unroll
                    for (int u = 0; u < BP; ++u)
                    {
                        fr[u] = ff_mul(K, pr[u]);
                        fi[u] = ff_mul(K, pi[u]);
                        r1[u] = {par ? 0.0f : 1.0f, 0.0f};
                        r0[u] = {0.0f, 0.0f};
                    }
                    for (int l = m0;; ++l)
                    {
                        if (((req >> l) & 1u) && l >= m)
                        {
                            float4* slot = my + (pb[l] + (m >> 1)) * T;
                            float4 v = *slot;
#pragma unroll
                            for (int u = 0; u < BP; ++u)
                            {
                                ff_acc(v.x, v.y, ff_mul(r1[u], fr[u]));
                                ff_acc(v.z, v.w, ff_mul(r1[u], fi[u]));
                            }
                            *slot = v;
                        }
                        if (l == lmax)
                            break;
                        const int mm = m <= ST_MAX_L ? m : ST_MAX_L;
                        const float2 af = c_aff[(l + 1) * (ST_MAX_L + 1) + mm];
                        const float2 bf = c_bff[(l + 1) * (ST_MAX_L + 1) + mm];
                        const bool start = l + 1 == m; // odd thread: R_m = 1
#pragma unroll
                        for (int u = 0; u < BP; ++u)
                        {
                            const ffl t = ff_sub_lazy(ff_mul(g[u].ct, r1[u]), ff_mul({bf.x, bf.y}, r0[u]));
                            const ffl nr = ff_mul({af.x, af.y}, t);
                            r0[u] = r1[u];
                            r1[u] = start ? ffl{1.0f, 0.0f} : nr;
                        }
                    }
                }
            }
        }
        // sums -> qlm (m of this parity) in place; ql from both threads' parts
        for (int kk = 0; kk < nl; ++kk)
        {
            const int l = s_lt[kk];
            float part = 0.0f;
            if (i < n)
            {
                for (int m = par; m <= l; m += 2)
                {
                    float4* slot = my + (pb[l] + (m >> 1)) * T;
                    const float4 v = *slot;
                    const float qr = ff_div_f(v.x, v.y, tw);
                    const float qi = ff_div_f(v.z, v.w, tw);
                    slot->x = qr;
                    slot->y = qi;
                    const float sq = __fmaf_rn(qr, qr, __fmul_rn(qi, qi));
                    part = __fadd_rn(part, m > 0 ? __fmul_rn(2.0f, sq) : sq);
                }
            }
            // even orders' part + odd orders' part (the same order on both threads)
            const float other = __shfl_xor_sync(FULL, part, 1);
            const float tot = par ? __fadd_rn(other, part) : __fadd_rn(part, other);
            if (i < n && par == 0)
                ql_out[static_cast<size_t>(i) * nl + s_k[kk]] = sqrtf(tot * s_norm[kk]);
        }
        __syncwarp();
        // the warp's 16 particles' rows, coalesced
        const uint32_t w0 = i0 + ((threadIdx.x & ~31u) >> 1);
        const int wcol = threadIdx.x & ~31;
        for (int kk = 0; kk < nl; ++kk)
        {
            const int l = s_lt[kk];
            const int width = 2 * l + 1;
            float2* out = qlm_out + s_off[kk] + static_cast<size_t>(w0) * width;
            for (int p = 0; p < 16 && w0 + p < n; ++p)
            {
                for (int c = lane; c < width; c += 32)
                {
                    const int m = c <= l ? c : c - l;
                    const float4 v = acc[(s_pb[m & 1][l] + (m >> 1)) * T + wcol + 2 * p + (m & 1)];
                    float2 q = make_float2(v.x, v.y);
                    if (c > l)
                        q = (m & 1) ? make_float2(-v.x, v.y) : make_float2(v.x, -v.y);
                    out[static_cast<size_t>(p) * width + c] = q;
                }
            }
        }
        __syncwarp();
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

// Neighbour averaging with the row entries of every l flattened: P lanes per
// particle, lane s owns entries s, s + P, ... of the E = sum (2l + 1) entries
// (each a fixed (l, column) of the per-l arrays), so one neighbour's whole row
// is R independent loads per lane, contiguous across the lanes. Sums run over
// the bonds in order, then the particle's own row, over (1 + n_i)
// (Steinhardt.cc:224-289), as k_ave; ql per l is a shuffle reduction of the
// lanes' squared magnitudes.
template<int P, int R>
__global__ void __launch_bounds__(128, 8)
    k_ave_flat(uint32_t n, const uint2* __restrict__ ij, const uint32_t* __restrict__ bj,
               const uint32_t* __restrict__ seg, const uint32_t* __restrict__ cnt, StLs ls, int E,
               const float2* __restrict__ qlm, float2* __restrict__ ave, float* __restrict__ ql_ave,
               const uint32_t* __restrict__ order)
{
    const int lane = threadIdx.x & 31;
    const int sub = lane % P;
    const int group = lane / P;
    const unsigned gmask = P == 32 ? FULL : (((1u << P) - 1u) << (group * P));
    const int gpb = blockDim.x / P;
    // entry r of this lane: column base pointer and row width (width 0 and the
    // array start for a lane past the last entry, whose sums are never used)
    const float2* col[R];
    uint32_t width[R];
    int kof[R];
#pragma unroll
    for (int r = 0; r < R; ++r)
    {
        const int e = sub + r * P;
        col[r] = qlm;
        width[r] = 0;
        kof[r] = -1;
        int start = 0;
        for (int k = 0; k < ls.nl; ++k)
        {
            const int w = 2 * ls.l[k] + 1;
            if (e >= start && e < start + w)
            {
                col[r] = qlm + ls.qlm_offset[k] + (e - start);
                width[r] = static_cast<uint32_t>(w);
                kof[r] = k;
            }
            start += w;
        }
    }
    for (uint32_t t = blockIdx.x * gpb + threadIdx.x / P; t < n; t += gridDim.x * gpb)
    {
        const uint32_t i = order != nullptr ? order[t] : t;
        const uint32_t b0 = seg[i];
        const uint32_t nbond = cnt[i];
        float sr[R], si[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
            sr[r] = si[r] = 0.0f;
        for (uint32_t base = 0; base < nbond; base += P)
        {
            const uint32_t jl =
                base + sub < nbond ? (bj != nullptr ? bj[b0 + base + sub] : ij[b0 + base + sub].y) : 0u;
            const uint32_t nh = min(static_cast<uint32_t>(P), nbond - base);
#pragma unroll 8
            for (uint32_t u = 0; u < nh; ++u)
            {
                const uint32_t j = __shfl_sync(gmask, jl, u, P);
#pragma unroll
                for (int r = 0; r < R; ++r)
                {
                    const float2 v = col[r][static_cast<size_t>(j) * width[r]];
                    sr[r] += v.x;
                    si[r] += v.y;
                }
            }
        }
        const float cntf = static_cast<float>(1u + nbond);
        float sq[R];
#pragma unroll
        for (int r = 0; r < R; ++r)
        {
            sq[r] = 0.0f;
            if (kof[r] >= 0)
            {
                const size_t a = static_cast<size_t>(i) * width[r];
                const float2 own = col[r][a];
                const float qr = (sr[r] + own.x) / cntf;
                const float qi = (si[r] + own.y) / cntf;
                ave[(col[r] - qlm) + a] = make_float2(qr, qi);
                sq[r] = qr * qr + qi * qi;
            }
        }
        for (int k = 0; k < ls.nl; ++k)
        {
            float part = 0.0f;
#pragma unroll
            for (int r = 0; r < R; ++r)
                part += kof[r] == k ? sq[r] : 0.0f;
            for (int o = P / 2; o > 0; o >>= 1)
                part += __shfl_xor_sync(gmask, part, o, P);
            if (sub == 0)
                ql_ave[static_cast<size_t>(i) * ls.nl + k] = sqrtf(part * ls.norm[k]);
        }
    }
}

// Wl per particle, every l of the set: thread per particle, the block's rows
// staged in shared memory (a straight copy: rows of consecutive particles are
// contiguous; the row length 2l + 1 is odd, so the rows' 8-byte reads are free of
// bank conflicts), the l's term classes broadcast from shared memory. Each class
// adds C x Re(q_a q_b q_c) in float-float (exact float products, TwoSum sums), so
// the sum is the FP64 triple sum of the float qlm to within about 2^-44 of its
// terms; it is rounded once, then normalised by (sqrt(4 pi / (2l + 1)) / ql)^3
// (Steinhardt.cc:338-352).
__device__ __forceinline__ ffl two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ ffl ff_mulf(ffl a, float b)
{
    const float p = __fmul_rn(a.h, b);
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return {p, e};
}

constexpr int WL_T = 128;

__global__ void __launch_bounds__(WL_T)
    k_wl(uint32_t n, StLs ls, WlTerms wt, const int4* __restrict__ terms, const float2* __restrict__ src,
         const float* __restrict__ qnorm, int normalize, float* __restrict__ wl_out)
{
    extern __shared__ float4 wl_smem[];
    const uint32_t i0 = blockIdx.x * WL_T;
    const uint32_t i = i0 + threadIdx.x;
    const uint32_t rows_here = min(static_cast<uint32_t>(WL_T), n - i0);
    for (int k = 0; k < ls.nl; ++k)
    {
        const int l = ls.l[k];
        const int width = 2 * l + 1;
        int4* s_terms = reinterpret_cast<int4*>(wl_smem);
        float2* rows = reinterpret_cast<float2*>(wl_smem + wt.cnt[k]);
        __syncthreads();
        for (int t = threadIdx.x; t < wt.cnt[k]; t += WL_T)
            s_terms[t] = terms[wt.off[k] + t];
        const float2* base = src + ls.qlm_offset[k] + static_cast<size_t>(i0) * width;
        for (uint32_t e = threadIdx.x; e < rows_here * width; e += WL_T)
            rows[e] = base[e];
        __syncthreads();
        if (i < n)
        {
            const char* row = reinterpret_cast<const char*>(rows + threadIdx.x * width);
            float ah = 0.0f, al = 0.0f;
#pragma unroll 2
            for (int t = 0; t < wt.cnt[k]; ++t)
            {
                const int4 rec = s_terms[t];
                const float2 qa = *reinterpret_cast<const float2*>(row + (rec.x & 0xffff));
                const float2 qb = *reinterpret_cast<const float2*>(row + (static_cast<unsigned>(rec.x) >> 16));
                const float2 qc = *reinterpret_cast<const float2*>(row + rec.y);
                const ffl ur = ff_sub_lazy(two_prod(qa.x, qb.x), two_prod(qa.y, qb.y));
                const ffl ui = ff_add_lazy(two_prod(qa.x, qb.y), two_prod(qa.y, qb.x));
                const ffl re = ff_sub_lazy(ff_mulf(ur, qc.x), ff_mulf(ui, qc.y));
                ff_acc(ah, al, ff_mul({__int_as_float(rec.z), __int_as_float(rec.w)}, re));
            }
            float sum = __fadd_rn(ah, al);
            if (normalize)
            {
                const float nf = sqrtf(ls.norm[k]) / qnorm[static_cast<size_t>(i) * ls.nl + k];
                sum *= nf * nf * nf;
            }
            wl_out[static_cast<size_t>(i) * ls.nl + k] = sum;
        }
    }
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
    // float-float tables: hi = RN(x), lo = RN(x - hi) of the FP64 value
    static float2 Kff[ST_MAX_L + 1];
    static float2 Aff[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    static float2 Bff[(ST_MAX_L + 1) * (ST_MAX_L + 1)];
    auto split = [](double x) {
        const float h = static_cast<float>(x);
        return make_float2(h, static_cast<float>(x - static_cast<double>(h)));
    };
    for (int m = 0; m <= L; ++m)
    {
        double lg = 0.5 * (std::log(2.0 * m + 1.0) - std::log(4.0 * M_PI) - std::lgamma(2.0 * m + 1.0));
        for (int t = 1; t <= m; ++t)
            lg += std::log(2.0 * t - 1.0);
        Kff[m] = split(((m & 1) ? -1.0 : 1.0) * std::exp(lg));
        for (int l = 0; l <= L; ++l)
        {
            double a = 0.0, bb = 0.0;
            if (l == m + 1)
            {
                a = std::sqrt(2.0 * m + 3.0);
            }
            else if (l >= m + 2)
            {
                a = std::sqrt((4.0 * l * l - 1.0) / (static_cast<double>(l) * l - static_cast<double>(m) * m));
                bb = std::sqrt(((l - 1.0) * (l - 1.0) - static_cast<double>(m) * m) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
            }
            Aff[l * (L + 1) + m] = split(a);
            Bff[l * (L + 1) + m] = split(bb);
        }
    }
    cudaMemcpyToSymbolAsync(c_Kff, Kff, sizeof(Kff), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_aff, Aff, sizeof(Aff), 0, cudaMemcpyHostToDevice, s);
    cudaMemcpyToSymbolAsync(c_bff, Bff, sizeof(Bff), 0, cudaMemcpyHostToDevice, s);
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

// slots per thread of k_qlm_ff2: requested (l, m) with m of the larger parity count
static size_t ff2_np(const StLs& ls)
{
    int o0 = 0, o1 = 0;
    for (int k = 0; k < ls.nl; ++k)
    {
        o0 += ls.l[k] / 2 + 1;
        o1 += (ls.l[k] + 1) / 2;
    }
    return static_cast<size_t>(o0 > o1 ? o0 : o1);
}

int qlm_ff_threads(const StLs& ls)
{
    int slots = 0;
    for (int k = 0; k < ls.nl; ++k)
        slots += ls.l[k] + 1;
    return slots <= 64 ? 64 : 32;
}

size_t qlm_ff_smem(const StLs& ls)
{
    int slots = 0;
    for (int k = 0; k < ls.nl; ++k)
        slots += ls.l[k] + 1;
    return static_cast<size_t>(slots) * qlm_ff_threads(ls) * sizeof(float4);
}

void launch_qlm(const DevBox& box, const float* pts, uint32_t n, const uint2* ij, const float* dist,
                const float* weights, const uint32_t* seg, const uint32_t* cnt, const StLs& ls, int weighted,
                float2* qlm, float* ql, cudaStream_t s, const float4* bond_vd, double mean_bonds, int precise)
{
    if (n == 0)
    {
        return;
    }
    if (precise)
    {
        const int T = qlm_ff_threads(ls);
        const size_t smem = qlm_ff_smem(ls);
        static bool configured = false;
        if (!configured)
        {
            // the largest set: ten l values up to 31
            const int most = 200 * 1024;
            cudaFuncSetAttribute(k_qlm_ff<64, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
            cudaFuncSetAttribute(k_qlm_ff<32, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
            configured = true;
        }
        // four bonds per pass: four independent recurrence chains per step
        // (0.85 ms against 0.99 ms with two on the 256,000-point FCC set, l = 4..12)
        if (ff2_np(ls) * 64 * sizeof(float4) <= 48 * 1024)
        {
            // two threads per particle (orders by parity): twice the particles per SM
            const uint32_t blocks2 = (n + 31) / 32;
            ProfScope prof2_("k_qlm_ff2", s);
            k_qlm_ff2<64, 4><<<blocks2, 64, ff2_np(ls) * 64 * sizeof(float4), s>>>(
                box, pts, n, ij, dist, weights, seg, cnt, bond_vd, ls, weighted, qlm, ql);
            return;
        }
        const uint32_t blocks = (n + T - 1) / T;
        ProfScope prof_("k_qlm_ff", s);
        auto go = [&](auto kernel, int threads) {
            kernel<<<blocks, threads, smem, s>>>(box, pts, n, ij, dist, weights, seg, cnt, bond_vd, ls, weighted, qlm,
                                                 ql);
        };
        if (T == 64)
            go(k_qlm_ff<64, 4>, 64);
        else
            go(k_qlm_ff<32, 4>, 32);
        return;
    }
    if (ls.nl == 1 && ls.max_l <= 12)
    {
        // one l: bonds flat over the lanes, about six rounds of 32 per warp group (64
        // uneven frames at density 0.85, r_max 1.5: 4.58 ms against 5.21 ms with three;
        // 4,096 Gaussian blobs, r_max 1.2: 1.57 against 1.53 ms)
        const double mb = mean_bonds > 0.0 ? mean_bonds : 24.0;
        const uint32_t per_warp = static_cast<uint32_t>(std::min(32.0, std::max(1.0, std::floor(192.0 / mb))));
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
    int E = 0;
    for (int k = 0; k < ls.nl; ++k)
        E += 2 * ls.l[k] + 1;
    const uint32_t cap = static_cast<uint32_t>(sm_count()) * 16;
    // rows of several l: flattened over the lanes (one l of up to 7 orders: the
    // order-per-lane kernel below is faster, 4.5 ms against 6.7 ms for l = 6 on the
    // 64 uneven frames)
    if (E > 16 && E <= 128)
    {
        const int P = 32;
        const uint32_t per_block = 128 / P;
        const uint32_t blocks = std::min<uint32_t>((n + per_block - 1) / per_block, cap);
        auto go = [&](auto kernel) {
            kernel<<<blocks, 128, 0, s>>>(n, ij, bond_j, seg, cnt, ls, E, qlm, ave, ql_ave, order);
        };
        ProfScope prof_("k_ave_flat", s);
        if (E <= 32)
            go(k_ave_flat<32, 1>);
        else if (E <= 64)
            go(k_ave_flat<32, 2>);
        else if (E <= 96)
            go(k_ave_flat<32, 3>);
        else
            go(k_ave_flat<32, 4>);
        return;
    }
    const int lanes = lanes_for(ls.max_l);
    const uint32_t groups = 128 / lanes;
    uint32_t blocks = (n + groups - 1) / groups;
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

std::vector<int4> wl_term_classes(int l, double (*w3j)(int, int, int, int))
{
    // class of (m1, m2, m3): its sorted members or those of its negation,
    // whichever sorts first; summed over the reference's index set
    std::vector<std::pair<std::array<int, 3>, double>> cls;
    for (int m1 = -l; m1 <= l; ++m1)
    {
        for (int m2 = std::max(-l - m1, -l); m2 <= std::min(l - m1, l); ++m2)
        {
            std::array<int, 3> t = {m1, m2, -m1 - m2};
            std::sort(t.begin(), t.end());
            std::array<int, 3> ng = {-t[2], -t[1], -t[0]};
            const std::array<int, 3> key = ng < t ? ng : t;
            auto it = std::find_if(cls.begin(), cls.end(), [&](const auto& c) { return c.first == key; });
            const double v = w3j(l, m1, m2, -m1 - m2);
            if (it == cls.end())
                cls.push_back({key, v});
            else
                it->second += v;
        }
    }
    std::vector<int4> out;
    for (const auto& c : cls)
    {
        // byte offset of each member's column in the row (m order 0..l, -1..-l)
        int col[3];
        for (int slot = 0; slot < 3; ++slot)
        {
            const int m = c.first[slot];
            col[slot] = 8 * (m >= 0 ? m : l - m);
        }
        const float h = static_cast<float>(c.second);
        const float lo = static_cast<float>(c.second - static_cast<double>(h));
        int4 r;
        r.x = col[0] | (col[1] << 16);
        r.y = col[2];
        std::memcpy(&r.z, &h, 4);
        std::memcpy(&r.w, &lo, 4);
        out.push_back(r);
    }
    return out;
}

void launch_wl(uint32_t n, const StLs& ls, const WlTerms& wt, const int4* terms, const float2* src,
               const float* qnorm, int normalize, float* wl, cudaStream_t s)
{
    if (n == 0)
    {
        return;
    }
    int most = 0;
    for (int k = 0; k < ls.nl; ++k)
        most = std::max(most, wt.cnt[k] * 16 + WL_T * (2 * ls.l[k] + 1) * 8);
    static bool configured = false;
    if (!configured)
    {
        // l = 31: 272 classes and 128 rows of 63 entries
        cudaFuncSetAttribute(k_wl, cudaFuncAttributeMaxDynamicSharedMemorySize, 80 * 1024);
        configured = true;
    }
    ProfScope prof_("k_wl", s);
    k_wl<<<(n + WL_T - 1) / WL_T, WL_T, most, s>>>(n, ls, wt, terms, src, qnorm, normalize, wl);
}


} // namespace fg
