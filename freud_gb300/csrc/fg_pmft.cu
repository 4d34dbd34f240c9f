// Potentials of mean force and torque (freud/pmft/PMFTR12.cc, PMFTXYT.cc,
// PMFTXY.cc, PMFTXYZ.cc): for every bond (query i, point j) with vector delta,
// coordinates in the query's frame are binned in a regular 2- or 3-axis
// histogram (Histogram.h:123-174, 301-351; row-major bins).
//
//   R12: (|delta|, t1, t2), t1 = mod+(theta_j - atan2(dy, dx), 2 pi),
//        t2 = mod+(theta_i - atan2(-dy, -dx), 2 pi)             (PMFTR12.cc:92-110)
//   XYT: (R(-theta_i) delta, mod+(theta_j - atan2(-dy, -dx), 2 pi)) (PMFTXYT.cc:79-100)
//   XY:  R(-theta_i) delta                                       (PMFTXY.cc:71-88)
//   XYZ: rotate(e_k, rotate(conj(q_i), delta)) for every equivalent
//        orientation e_k                                         (PMFTXYZ.cc:116-145)
//
// Float arithmetic follows the reference's operation order with explicit
// rounding (no contraction). R(-theta) comes from cos/sin computed on the host
// with the C library, as the reference computes them; atan2 runs on the device
// (CUDA's atan2f), so a bond within an ulp of a bin edge in t may fall in the
// neighbouring bin. Counts are uint64 in global memory (histograms of up to
// millions of bins).
#include "fg_common.cuh"
#include "fg_kernels.cuh"
#include "fg_prof.cuh"

namespace fg {

namespace {

constexpr float TWO_PI_F = 6.2831854820251465f; // float(2 pi), as the reference's constant

__device__ __forceinline__ uint32_t axis_bin(float v, const PmftAxis& a)
{
    // RegularAxis::bin (Histogram.h:152-174): out of [min, max) -> overflow sentinel
    if (v < a.min || v >= a.max)
        return 0xffffffffu;
    const float val = __fmul_rn(__fsub_rn(v, a.min), a.inv);
    uint32_t b = static_cast<uint32_t>(val);
    if (b == a.n)
        b = a.n - 1;
    return b;
}

// util::modulusPositive(a, 2 pi) = fmod(fmod(a, b) + b, b) (utils.h:29-32); fmodf is exact
__device__ __forceinline__ float mod_two_pi(float a)
{
    return fmodf(__fadd_rn(fmodf(a, TWO_PI_F), TWO_PI_F), TWO_PI_F);
}

struct Q4
{
    float s, x, y, z;
};

// rotate(quat, vec3) (VectorMath.h:810-823):
// (s*s - dot(v, v)) * b + 2 * s * cross(v, b) + 2 * dot(v, b) * v
__device__ __forceinline__ void qrotate(const Q4& a, float bx, float by, float bz, float& ox, float& oy, float& oz)
{
    const float vv = __fadd_rn(__fadd_rn(__fmul_rn(a.x, a.x), __fmul_rn(a.y, a.y)), __fmul_rn(a.z, a.z));
    const float t1 = __fsub_rn(__fmul_rn(a.s, a.s), vv);
    const float s2 = __fmul_rn(2.0f, a.s);
    const float cx = __fsub_rn(__fmul_rn(a.y, bz), __fmul_rn(a.z, by));
    const float cy = __fsub_rn(__fmul_rn(a.z, bx), __fmul_rn(a.x, bz));
    const float cz = __fsub_rn(__fmul_rn(a.x, by), __fmul_rn(a.y, bx));
    const float vb = __fadd_rn(__fadd_rn(__fmul_rn(a.x, bx), __fmul_rn(a.y, by)), __fmul_rn(a.z, bz));
    const float d2 = __fmul_rn(2.0f, vb);
    ox = __fadd_rn(__fadd_rn(__fmul_rn(t1, bx), __fmul_rn(s2, cx)), __fmul_rn(d2, a.x));
    oy = __fadd_rn(__fadd_rn(__fmul_rn(t1, by), __fmul_rn(s2, cy)), __fmul_rn(d2, a.y));
    oz = __fadd_rn(__fadd_rn(__fmul_rn(t1, bz), __fmul_rn(s2, cz)), __fmul_rn(d2, a.z));
}

template<int KIND>
__global__ void k_pmft_bonds(const uint2* __restrict__ ij, const float* __restrict__ dist,
                             const float* __restrict__ vec, uint64_t nb, const float* __restrict__ p_angle,
                             const float* __restrict__ q_angle, const float2* __restrict__ q_cs,
                             const float4* __restrict__ q_quat, const float4* __restrict__ equiv, PmftParams pp,
                             unsigned long long* __restrict__ hist)
{
    const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < nb; e += stride)
    {
        const uint2 b = ij[e];
        const float dx = vec[3 * e], dy = vec[3 * e + 1], dz = vec[3 * e + 2];
        if (KIND == PMFT_R12)
        {
            const float th1 = atan2f(dy, dx);
            const float th2 = atan2f(-dy, -dx);
            const float t1 = mod_two_pi(__fsub_rn(p_angle[b.y], th1));
            const float t2 = mod_two_pi(__fsub_rn(q_angle[b.x], th2));
            const uint32_t b0 = axis_bin(dist[e], pp.ax[0]);
            const uint32_t b1 = axis_bin(t1, pp.ax[1]);
            const uint32_t b2 = axis_bin(t2, pp.ax[2]);
            if (b0 != 0xffffffffu && b1 != 0xffffffffu && b2 != 0xffffffffu)
                atomicAdd(&hist[(static_cast<uint64_t>(b0) * pp.ax[1].n + b1) * pp.ax[2].n + b2], 1ull);
        }
        else if (KIND == PMFT_XYT || KIND == PMFT_XY)
        {
            // rotmat2::fromAngle(-theta_i) * (dx, dy) (VectorMath.h:912-921, 934-937)
            const float2 cs = q_cs[b.x]; // (cos(-theta_i), sin(-theta_i))
            const float rx = __fadd_rn(__fmul_rn(cs.x, dx), __fmul_rn(-cs.y, dy));
            const float ry = __fadd_rn(__fmul_rn(cs.y, dx), __fmul_rn(cs.x, dy));
            const uint32_t b0 = axis_bin(rx, pp.ax[0]);
            const uint32_t b1 = axis_bin(ry, pp.ax[1]);
            if (b0 == 0xffffffffu || b1 == 0xffffffffu)
                continue;
            if (KIND == PMFT_XY)
            {
                atomicAdd(&hist[static_cast<uint64_t>(b0) * pp.ax[1].n + b1], 1ull);
            }
            else
            {
                const float t = mod_two_pi(__fsub_rn(p_angle[b.y], atan2f(-dy, -dx)));
                const uint32_t b2 = axis_bin(t, pp.ax[2]);
                if (b2 != 0xffffffffu)
                    atomicAdd(&hist[(static_cast<uint64_t>(b0) * pp.ax[1].n + b1) * pp.ax[2].n + b2], 1ull);
            }
        }
        else
        {
            const float4 qq = q_quat[b.x];
            const Q4 cq {qq.x, -qq.y, -qq.z, -qq.w}; // conj(q_i): (s, -v)
            float ux, uy, uz;
            qrotate(cq, dx, dy, dz, ux, uy, uz);
            for (uint32_t k = 0; k < pp.n_equiv; ++k)
            {
                const float4 ek = equiv[k];
                float vx, vy, vz;
                qrotate(Q4 {ek.x, ek.y, ek.z, ek.w}, ux, uy, uz, vx, vy, vz);
                const uint32_t b0 = axis_bin(vx, pp.ax[0]);
                const uint32_t b1 = axis_bin(vy, pp.ax[1]);
                const uint32_t b2 = axis_bin(vz, pp.ax[2]);
                if (b0 != 0xffffffffu && b1 != 0xffffffffu && b2 != 0xffffffffu)
                    atomicAdd(&hist[(static_cast<uint64_t>(b0) * pp.ax[1].n + b1) * pp.ax[2].n + b2], 1ull);
            }
        }
    }
}

} // namespace

void launch_pmft_bonds(int kind, const uint2* ij, const float* dist, const float* vec, uint64_t nb,
                       const float* p_angle, const float* q_angle, const float2* q_cs, const float4* q_quat,
                       const float4* equiv, const PmftParams& pp, unsigned long long* hist, cudaStream_t s)
{
    if (nb == 0)
        return;
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (nb + 255) / 256;
    const uint64_t cap = static_cast<uint64_t>(sms) * 8;
    const unsigned blocks = static_cast<unsigned>(want < cap ? want : cap);
    ProfScope prof_("k_pmft_bonds", s);
    switch (kind)
    {
    case PMFT_R12:
        k_pmft_bonds<PMFT_R12><<<blocks, 256, 0, s>>>(ij, dist, vec, nb, p_angle, q_angle, q_cs, q_quat, equiv, pp,
                                                       hist);
        break;
    case PMFT_XYT:
        k_pmft_bonds<PMFT_XYT><<<blocks, 256, 0, s>>>(ij, dist, vec, nb, p_angle, q_angle, q_cs, q_quat, equiv, pp,
                                                       hist);
        break;
    case PMFT_XY:
        k_pmft_bonds<PMFT_XY><<<blocks, 256, 0, s>>>(ij, dist, vec, nb, p_angle, q_angle, q_cs, q_quat, equiv, pp,
                                                      hist);
        break;
    default:
        k_pmft_bonds<PMFT_XYZ><<<blocks, 256, 0, s>>>(ij, dist, vec, nb, p_angle, q_angle, q_cs, q_quat, equiv, pp,
                                                       hist);
        break;
    }
}

} // namespace fg
