// Mixed-precision phase evaluation shared by the pointwise, batched and
// adjoint kernels (phases taken relative to an origin point, see
// rotate_to_origin below).
//
// The phase in turns t = <q, x> with q = k / (2 pi) is reduced modulo 1
// without FP64 arithmetic per (mode, point):
//   * q and x are split into a head with at most 12 significant bits and an
//     FP32 tail (q = qh + ql, x = xh + xl, xf = fp32(x));
//   * qh * xh is exact in FP32 (12 x 12 bits), so its integer part can be
//     removed exactly with the 1.5 * 2^23 rounding trick (|qh xh| < 2^22);
//   * the small cross terms qh * xl + ql * xf carry the rest;
//   * the sum is reduced once more to [-1/2, 1/2] turns.
// The reduced angle then feeds the SFU sin/cos.  Phase error is about
// 2^-24 + |t| 2^-35 turns; per-axis domain |q_d x_d| < 2^21 turns.
#pragma once

#include "gst_common.cuh"

namespace gst {

constexpr float kRoundMagicF = 12582912.0f;  // 1.5 * 2^23
constexpr float kTwoPiF = 6.28318530717958647692f;

template <int DIM>
struct MixedPoint {
    float xh[DIM], xl[DIM], xf[DIM];
};

template <int DIM>
__device__ __forceinline__ MixedPoint<DIM> mixed_split_point(const double (&x)[DIM]) {
    MixedPoint<DIM> p;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        p.xh[d] = split_hi12(x[d]);
        p.xl[d] = static_cast<float>(x[d] - static_cast<double>(p.xh[d]));
        p.xf[d] = static_cast<float>(x[d]);
    }
    return p;
}

// Reduced phase (turns, in [-1/2, 1/2]) of one mode / point pair.
template <int DIM>
__device__ __forceinline__ float mixed_turns(const float (&qh)[3],
                                             const float (&ql)[3],
                                             const MixedPoint<DIM> &p) {
    float r = 0.0f, cross = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const float prod = __fmul_rn(qh[d], p.xh[d]);
        const float nint = __fsub_rn(__fadd_rn(prod, kRoundMagicF), kRoundMagicF);
        const float frac = __fsub_rn(prod, nint);
        r = (d == 0) ? frac : __fadd_rn(r, frac);
        cross = fmaf(qh[d], p.xl[d], cross);
        cross = fmaf(ql[d], p.xf[d], cross);
    }
    r = __fadd_rn(r, cross);
    return __fsub_rn(r, __fsub_rn(__fadd_rn(r, kRoundMagicF), kRoundMagicF));
}

// Reduced turns of <q, x> - psi (psi in [-1/2, 1/2]), in [-1/2, 1/2]: the
// split reduction above with psi folded into the cross terms.
template <int DIM>
__device__ __forceinline__ float mixed_turns_minus(const float (&qh)[3],
                                                   const float (&ql)[3],
                                                   const MixedPoint<DIM> &p,
                                                   float psi) {
    float r = 0.0f, cross = -psi;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const float prod = __fmul_rn(qh[d], p.xh[d]);
        const float nint = __fsub_rn(__fadd_rn(prod, kRoundMagicF), kRoundMagicF);
        const float frac = __fsub_rn(prod, nint);
        r = (d == 0) ? frac : __fadd_rn(r, frac);
        cross = fmaf(qh[d], p.xl[d], cross);
        cross = fmaf(ql[d], p.xf[d], cross);
    }
    r = __fadd_rn(r, cross);
    return __fsub_rn(r, __fsub_rn(__fadd_rn(r, kRoundMagicF), kRoundMagicF));
}

template <int DIM>
__device__ __forceinline__ void mixed_sincos(const float (&qh)[3],
                                             const float (&ql)[3],
                                             const MixedPoint<DIM> &p,
                                             float *sn, float *cs) {
    __sincosf(mixed_turns<DIM>(qh, ql, p) * kTwoPiF, sn, cs);
}

// Origin shift of the mixed paths: with x = x0 + x' and theta = <k, x>,
//   a1 cos(theta) + a2 sin(theta) = a1' cos(<k, x'>) + a2' sin(<k, x'>),
//   a1' = a1 cos(a) + a2 sin(a),  a2' = a2 cos(a) - a1 sin(a),  a = <k, x0>,
// so the per-point phases span only the extent of the points around x0 (the
// split turn reduction's error grows with |<k, x>|).  The rotation is formed
// once per mode: <k, x0> / 2 pi reduced exactly in FP64, the sincospi of the
// reduced angle in FP32.  A coordinate of x0 that is not finite is taken as 0.
__device__ __forceinline__ double origin_coord(const double *p) {
    if (p == nullptr) return 0.0;
    const double v = *p;
    return isfinite(v) ? v : 0.0;
}

__device__ __forceinline__ void rotate_to_origin(const double (&k)[4], int dim,
                                                 const double (&x0)[3], double &a1,
                                                 double &a2) {
    constexpr double kInv2PiD = 0.15915494309189533576888376337251436;
    double t = 0.0;
    for (int d = 0; d < dim && d < 3; ++d) t += (k[d] * kInv2PiD) * x0[d];
    const double r = t - rint(t);   // exact, |r| <= 1/2
    // FP32 sincospi of the reduced angle: the rotated amplitudes are rounded
    // to FP32 in the table anyway (an FP64 sincospi per mode was measured to
    // add 1.5 % to a 1000-mode x 100 000-point call)
    float sf, cf;
    sincospif(2.0f * static_cast<float>(r), &sf, &cf);
    const double s = sf, c = cf;
    const double b1 = a1 * c + a2 * s;
    const double b2 = a2 * c - a1 * s;
    a1 = b1;
    a2 = b2;
}

// Packs one mode into the 16-float mixed table entry
//   qh0 qh1 qh2 a1 | ql0 ql1 ql2 a2 | p0 p1 p2 0 | 0 0 0 0
__device__ __forceinline__ void mixed_pack_entry(float *e, const double (&k)[4],
                                                 double a1, double a2,
                                                 const double (&proj)[3]) {
    constexpr double kInv2Pi = 0.15915494309189533576888376337251436;
    for (int d = 0; d < 3; ++d) {
        const double q = k[d] * kInv2Pi;
        const float qh = split_hi12(q);
        e[d] = qh;
        e[4 + d] = static_cast<float>(q - static_cast<double>(qh));
        e[8 + d] = static_cast<float>(proj[d]);
    }
    e[3] = static_cast<float>(a1);
    e[7] = static_cast<float>(a2);
    for (int d = 11; d < 16; ++d) e[d] = 0.0f;
}

}  // namespace gst
