// Shared device/host definitions for the freud_gb300 CUDA library.
//
// Exact float32 box arithmetic: every operation that decides a neighbour set,
// a bond vector, a distance or an RDF bin uses the explicitly rounded intrinsics
// (__fadd_rn, __fsub_rn, __fmul_rn, __fdiv_rn, __fsqrt_rn) so nvcc cannot contract
// them into FMAs. The order of operations follows freud/box/Box.h:212-329 and
// freud/util/VectorMath.h:270-273, which makes the results bit-identical to the
// reference's x86-64 build.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fg {

constexpr int WARP = 32;

// Device view of a periodic box (freud::box::Box with all three periodic flags set).
struct DevBox
{
    float L[3];   // Lx, Ly, Lz (Lz = 0 in 2D)
    float lo[3];  // -L/2
    float xy, xz, yz;
    int is2d;
    float img[27][3]; // reference image vectors, index (kx+1)*9 + (ky+1)*3 + (kz+1)
    float rcp[3];     // RN(1 / L) per axis (0 where L = 0), for div_rn_recip
    int tilted;       // nonzero when any of xy, xz, yz is nonzero
};

__host__ __device__ inline float fadd(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}
__host__ __device__ inline float fsub(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
__host__ __device__ inline float fmul(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}
__host__ __device__ inline float fdiv(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    volatile float r = a / b;
    return r;
#endif
}

// (x*x + y*y) + z*z, VectorMath.h:270-273
__device__ __forceinline__ float dot3(float x, float y, float z)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

// fmodf(a, 1.0f) is exactly a - truncf(a): the fractional part of a float is
// representable, so the subtraction is exact (also for |a| >= 2^23 and +-0).
__device__ __forceinline__ float fmod1(float a)
{
    return __fsub_rn(a, truncf(a));
}

// a / b rounded to nearest even, given y = RN(1 / b), for a != -0 and a / b
// normal or zero (the box arithmetic divides coordinates by box lengths: no
// overflow or underflow). q0 = RN(a y) is within 1.5 ulp of a / b; one
// correction q1 = RN(q0 + (a - b q0) y) (fused, so the residual enters
// unrounded) brings it within one ulp; from a q1 within one ulp and
// y = RN(1 / b), Markstein's theorem (P. Markstein, IBM J. Res. Dev. 34(1),
// 1990; Muller et al., Handbook of Floating-Point Arithmetic, the theorem on
// correcting a quotient with the exact FMA remainder) makes q1 + (a - b q1) y,
// rounded once, the correctly rounded quotient. a = +0 gives +0 at every step.
// The box arithmetic divides v - lo with lo != 0, which is never -0 in
// round-to-nearest (x - y is -0 only for x = -0, y = +0).
__device__ __forceinline__ float div_rn_recip_nz(float a, float b, float y)
{
    const float q0 = __fmul_rn(a, y);
    const float q1 = __fmaf_rn(__fmaf_rn(-q0, b, a), y, q0);
    return __fmaf_rn(__fmaf_rn(-q1, b, a), y, q1);
}

// The same for any a: a = -0 returns a * y = -0 (the corrections would turn it
// into +0).
__device__ __forceinline__ float div_rn_recip(float a, float b, float y)
{
    return a == 0.0f ? __fmul_rn(a, y) : div_rn_recip_nz(a, b, y);
}

// util::modulusPositive(a, 1.0f) = fmod(fmod(a, 1) + 1, 1), utils.h:29-32
__device__ __forceinline__ float mod_pos1(float a)
{
    return fmod1(__fadd_rn(fmod1(a), 1.0f));
}

// Box::makeFractional, Box.h:243-255. In a box without tilt the tilt terms are
// +-0 and subtracting them changes nothing (for finite v): dx = v - lo is never
// -0 because lo != 0, so they are skipped there. Divisions by the box lengths are
// correctly rounded (div_rn_recip_nz: v - lo is never -0), so the quotients equal
// IEEE division's.
__device__ __forceinline__ void make_fractional(const DevBox& b, float vx, float vy, float vz, float& fx,
                                                float& fy, float& fz)
{
    float dx = __fsub_rn(vx, b.lo[0]);
    float dy = __fsub_rn(vy, b.lo[1]);
    float dz = __fsub_rn(vz, b.lo[2]);
    if (b.tilted)
    {
        const float t2 = __fsub_rn(b.xz, __fmul_rn(b.yz, b.xy));
        dx = __fsub_rn(dx, __fadd_rn(__fmul_rn(t2, vz), __fmul_rn(b.xy, vy)));
        dy = __fsub_rn(dy, __fmul_rn(b.yz, vz));
    }
    fx = div_rn_recip_nz(dx, b.L[0], b.rcp[0]);
    fy = div_rn_recip_nz(dy, b.L[1], b.rcp[1]);
    fz = b.is2d ? 0.0f : div_rn_recip_nz(dz, b.L[2], b.rcp[2]);
}

// Box::makeAbsolute, Box.h:212-222 (tilt terms skipped in a box without tilt:
// x + (+-0) = x for finite x, and x = lo + f L is never -0)
__device__ __forceinline__ void make_absolute(const DevBox& b, float fx, float fy, float fz, float& x, float& y,
                                              float& z)
{
    x = __fadd_rn(b.lo[0], __fmul_rn(fx, b.L[0]));
    y = __fadd_rn(b.lo[1], __fmul_rn(fy, b.L[1]));
    z = __fadd_rn(b.lo[2], __fmul_rn(fz, b.L[2]));
    if (b.tilted)
    {
        x = __fadd_rn(x, __fadd_rn(__fmul_rn(b.xy, y), __fmul_rn(b.xz, z)));
        y = __fadd_rn(y, __fmul_rn(b.yz, z));
    }
    if (b.is2d)
    {
        z = 0.0f;
    }
}

// Box::wrap for a fully periodic box, Box.h:307-329
__device__ __forceinline__ void box_wrap(const DevBox& b, float vx, float vy, float vz, float& x, float& y,
                                         float& z)
{
    float fx, fy, fz;
    make_fractional(b, vx, vy, vz, fx, fy, fz);
    make_absolute(b, mod_pos1(fx), mod_pos1(fy), mod_pos1(fz), x, y, z);
}

__device__ __forceinline__ int pack_image(int nx, int ny, int nz)
{
    return (nx & 0xff) | ((ny & 0xff) << 8) | ((nz & 0xff) << 16);
}

__device__ __forceinline__ int clamp_img(float n)
{
    return n < -100.0f ? -100 : (n > 100.0f ? 100 : static_cast<int>(n));
}

// One axis of a packed integer box image (signed 8 bits per axis).
__device__ __forceinline__ int img_ax(int bits, int axis)
{
    return static_cast<int>(static_cast<int8_t>((bits >> (8 * axis)) & 0xff));
}

// Wrapped cell coordinate and integer image of a point (fractional coordinate
// f = n + u with n = floor(f), u in [0, 1)).
__device__ __forceinline__ void point_cell(const DevBox& b, const int dim[3], float x, float y, float z,
                                           int& cx, int& cy, int& cz, int& img)
{
    float fx, fy, fz;
    make_fractional(b, x, y, z, fx, fy, fz);
    const float nx = floorf(fx);
    const float ny = floorf(fy);
    const float nz = floorf(fz);
    const float ux = __fsub_rn(fx, nx);
    const float uy = __fsub_rn(fy, ny);
    const float uz = __fsub_rn(fz, nz);
    cx = min(static_cast<int>(ux * static_cast<float>(dim[0])), dim[0] - 1);
    cy = min(static_cast<int>(uy * static_cast<float>(dim[1])), dim[1] - 1);
    cz = b.is2d ? 0 : min(static_cast<int>(uz * static_cast<float>(dim[2])), dim[2] - 1);
    cx = max(cx, 0);
    cy = max(cy, 0);
    cz = max(cz, 0);
    img = pack_image(clamp_img(nx), clamp_img(ny), b.is2d ? 0 : clamp_img(nz));
}

// Error word written by kernels whose waits or capacities are bounded.
enum DeviceError : int
{
    DEV_OK = 0,
    DEV_CAPACITY = 1,  // a per-query staging buffer overflowed
    DEV_TIMEOUT = 2,   // a bounded spin gave up
    DEV_RANGE = 3,     // an index fell outside its buffer (debug checks)
};

} // namespace fg
