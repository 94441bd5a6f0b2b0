// kernels.cuh -- the solve-path kernels for sm_103a, templated on the stencil
// precision T (double or float).
//
// One RK stage is four passes over the cells (a grid-wide dependency
// separates each pair):
//   A  k_faces : boundary ghosts + Green-Gauss gradient + neighbour min/max
//                + per-face limited reconstruction of the cell's own side of
//                its three faces + spectral radius sum -> local time step
//   B  k_flux  : per cell, Roe flux of its three faces from the two face-side
//                states, summed with the reference's signs and face order
//   C  k_smooth: implicit residual smoothing sweep (all but the last sweep)
//   D  k_update: last smoothing sweep + magnitude clamp + RK update, and on
//                the last stage the (rho - rho0)^2 block partials
// and k_resid folds the partials into Resd on the last stage.
//
// Every cell gathers its own faces, so nothing is accumulated with atomics
// and the result does not depend on scheduling.  An interior face inside one
// block's tile of cells is evaluated once; a face between two tiles is
// evaluated by both cells from identical inputs, so both see the same value.  The arithmetic of each quantity follows the reference kernel
// it replaces operation by operation (cited per function); compiled without
// FMA contraction, the FP64 instantiation reproduces the CPU oracle bit for
// bit.
#pragma once

#include "dev_types.h"
#include "pdl.cuh"

namespace e2d {

// Occupancy targets (minimum resident 256-thread blocks per SM) of the two
// gather kernels; the register budget follows from them.  Build-time knobs.
// 0 leaves the choice to the compiler.  Both kernels are latency bound.
// Pass A: 6 (40 registers); on the 4.2M-cell mesh 6 beat the compiler's own
// 48-register choice by 12 % (sweep over 1, 4, 5, 6 at 128 and 256 threads
// per block).  Pass B requests the inputs of all three faces before its
// first flux, which needs 63 registers: 4 blocks (99.7 -> 89.2 us per launch
// against the one-face-at-a-time form at 6 blocks; 94.4 us at 5 blocks,
// where it spills).
#ifndef E2D_MINB_FACES
#define E2D_MINB_FACES 6
#endif
#ifndef E2D_MINB_FLUX
#define E2D_MINB_FLUX 4
#endif
// The targets apply to the FP32 kernels; the FP64 (parity) kernels keep two
// blocks, enough registers for their ~100 live doubles without spilling.
template <typename T> struct MinBlocks { static constexpr int faces = 2, flux = 2; };
template <> struct MinBlocks<float> {
    static constexpr int faces = E2D_MINB_FACES > 0 ? E2D_MINB_FACES : 1;
    static constexpr int flux = E2D_MINB_FLUX > 0 ? E2D_MINB_FLUX : 1;
};
#define E2D_LB_FACES __launch_bounds__(256, MinBlocks<T>::faces)
// The batched (persistent, tile-walking) FP32 kernels hold a few more live
// values across their tile loop: one block fewer per SM, so that they do not
// spill (at the single-case targets ptxas spilled 144 / 60 bytes per thread).
template <typename T> struct BatchMinBlocks {
    static constexpr int faces = MinBlocks<T>::faces > 2 ? MinBlocks<T>::faces - 1 : MinBlocks<T>::faces;
    static constexpr int flux = MinBlocks<T>::flux > 2 ? MinBlocks<T>::flux - 1 : MinBlocks<T>::flux;
};

// Pass B variant.  FP64 evaluates each interior face inside a block's tile of
// cells once (flux_tile): the FP64 Roe flux is arithmetic bound on this GPU,
// and evaluating about half as many cut a whole FP64 iteration on a 51.8k-cell
// mesh from 1.75 to 1.27 ms.  FP32 is bound by memory latency, where the
// tile's work list and barriers cost more than they save (0.152 against
// 0.110 ms per launch on 4.2M cells), so every cell evaluates its own three
// faces (flux_cell).  Either way both cells of a face use the same flux bits.
template <typename T> struct FluxTiled { static constexpr bool value = sizeof(T) == 8; };
#define E2D_LB_FLUX __launch_bounds__(256, MinBlocks<T>::flux)

template <typename T> __device__ __forceinline__ T tabs(T v) { return fabs(v); }
template <typename T> __device__ __forceinline__ T tsqrt(T v) { return sqrt(v); }
template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return fmin(a, b); }
template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return fmax(a, b); }

// a * b + c: two roundings in FP64 (the oracle's arithmetic; the FP64 units
// are built without contraction), one fused multiply-add in FP32.  Explicit,
// so the FP32 result does not depend on where the compiler contracts.
template <typename T> __device__ __forceinline__ T madd(T a, T b, T c) { return a * b + c; }
template <> __device__ __forceinline__ float madd<float>(float a, float b, float c) { return fmaf(a, b, c); }

// Divisions and square roots of the stencil's hot paths: IEEE in FP64 (bit
// parity with the oracle); in FP32 the special-function unit's approximate
// reciprocal, reciprocal square root and square root (rcp / rsqrt /
// sqrt.approx.f32, a few ulp), one instruction each where the IEEE forms take
// a refinement sequence: the FP32 gather passes are issue bound.
__device__ __forceinline__ float frcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float frsqrt(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float fsqrt(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
template <typename T> __device__ __forceinline__ T fdiv(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float fdiv<float>(float a, float b) { return a * frcp(b); }

template <typename T> __device__ __forceinline__ T comp(const V4<T> &v, int k) {
    return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w;
}

// gpu_solver.cu:49-60 (kernel_CalculationPTA): pressure and sound speed
template <typename T> __device__ __forceinline__ void pta(const V4<T> &w, T g, T &P, T &A) {
    T U = w.y / w.x;
    T V = w.z / w.x;
    T E = w.w / w.x - T(0.5) * (U * U + V * V);
    P = (g - T(1.0)) * w.x * E;
    A = tsqrt(g * P / w.x);
}

// gpu_solver.cu:62-135 (kernel_Far_Boundary): far-field ghost state from the
// interior state dw (with its P, A) and the face vector (vectorx, vectory).
template <typename T>
__device__ __noinline__ V4<T> far_ghost(const V4<T> dw, T P, T A, T vectorx, T vectory,
                                        const Flow<T> f) {
    const T g = f.gamma;
    T nn = tsqrt(vectorx * vectorx + vectory * vectory);
    T nx = vectory / nn;
    T ny = vectorx / nn;
    T UD = dw.y / dw.x;
    T VD = dw.z / dw.x;
    T Un = tabs(f.ui * nx + f.vi * ny);
    T Uncell = UD * nx + VD * ny;
    V4<T> w0 = dw;
    if (Un / f.ain > T(1.0)) {
        if (!(Uncell > T(0.0))) {
            w0.x = T(1.0);
            w0.y = f.ui;
            w0.z = f.vi;
            w0.w = f.R * f.tin / (f.vin * f.vin) / (g - T(1.0)) + T(0.50);
        }
    } else {
        T PA = f.pis, PD = P, AD = A, ROUD = dw.x, PB, UB, VB;
        if (Uncell > T(0.0)) {
            PB = PA;
            w0.x = ROUD + (PB - PD) / AD / AD;
            UB = UD + nx * (PD - PB) / ROUD / AD;
            VB = VD + ny * (PD - PB) / ROUD / AD;
        } else {
            PB = T(0.5) * (PA + PD - ROUD * AD * (nx * (f.ui - UD) + ny * (f.vi - VD)));
            w0.x = T(1.0) + (PB - PA) / AD / AD;
            UB = f.ui - nx * (PA - PB) / ROUD / AD;
            VB = f.vi - ny * (PA - PB) / ROUD / AD;
        }
        w0.y = UB * w0.x;
        w0.z = VB * w0.x;
        w0.w = PB / (g - T(1.0)) + T(0.5) * (UB * UB + VB * VB) * w0.x;
    }
    return w0;
}

// gpu_solver.cu:188-221: slip-wall ghost (velocity mirrored in the face)
template <typename T>
__device__ __forceinline__ V4<T> wall_ghost(const V4<T> &dw, T vectorx, T vectory, T vectorn) {
    T nij0 = vectory / vectorn;
    T nij1 = vectorx / vectorn;
    T UU = dw.y / dw.x;
    T VV = dw.z / dw.x;
    T UV = UU * nij0 + VV * nij1;
    UU = UU - T(2) * UV * nij0;
    VV = VV - T(2) * UV * nij1;
    V4<T> o = dw;
    o.y = dw.x * UU;
    o.z = dw.x * VV;
    return o;
}

// Ghost state across a boundary face code (-1 far, -2 wall).
template <typename T>
__device__ __forceinline__ V4<T> ghost(int code, const V4<T> &U, T Sx, T Sy, const Flow<T> &f) {
    if (code == -1) {
        T P, A;
        pta(U, f.gamma, P, A);
        return far_ghost(U, P, A, Sy, Sx, f);
    }
    T vn = tsqrt(Sy * Sy + Sx * Sx);
    return wall_ghost(U, Sy, Sx, vn);
}

// gpu_solver.cu:385-454 (kernel_deltT): face spectral radius from the mean of
// the two unreconstructed states.  Symmetric in (a, b) and in the sign of S.
template <typename T>
__device__ __forceinline__ T spectral_radius(const V4<T> &a, const V4<T> &b, T vectorx, T vectory,
                                             T g) {
    T rou = (a.x + b.x) * T(0.5);
    T u = (a.y + b.y) / rou * T(0.5);
    T v = (a.z + b.z) / rou * T(0.5);
    T EE = (a.w + b.w) * T(0.5) / rou - (u * u + v * v) * T(0.5);
    T VC = u * vectory + v * vectorx;
    T p = rou * EE * (g - T(1.0));
    T CS = tsqrt((g * p / rou) * (vectorx * vectorx + vectory * vectory));
    return tabs(VC) + CS;
}

// FP32: the same quantity with one reciprocal and fused multiply-adds.
template <>
__device__ __forceinline__ float spectral_radius<float>(const V4<float> &a, const V4<float> &b, float vectorx,
                                                       float vectory, float g) {
    const float2 s01 = __fadd2_rn(make_float2(a.x, a.y), make_float2(b.x, b.y));
    const float2 s23 = __fadd2_rn(make_float2(a.z, a.w), make_float2(b.z, b.w));
    const float rou = s01.x * 0.5f, ir = frcp(rou);
    const float u = s01.y * (0.5f * ir), v = s23.x * (0.5f * ir);
    const float EE = fmaf(s23.y * 0.5f, ir, -0.5f * fmaf(u, u, v * v));
    const float VC = fmaf(u, vectory, v * vectorx);
    const float p = rou * EE * (g - 1.0f);
    const float CS = fsqrt(g * p * ir * fmaf(vectorx, vectorx, vectory * vectory));
    return fabsf(VC) + CS;
}

// gpu_solver.cu:552-566 (kernel_Calc_Function)
template <typename T>
__device__ __forceinline__ void calc_function(const V4<T> &w, T g, T &A, T &U, T &V, T &H, T &P) {
    T temp = T(1.0) / w.x;
    U = w.y * temp;
    V = w.z * temp;
    P = (g - T(1.0)) * w.x * (w.w * temp - T(0.5) * (U * U + V * V));
    A = tsqrt(g * P * temp);
    H = w.w * temp + P * temp;
}

// gpu_solver.cu:569-647 (kernel_ROE_SCHEME): Roe flux with Harten's entropy
// fix of width eps through the unit normal (nx, ny).
template <typename T>
__device__ __forceinline__ V4<T> roe(const V4<T> &LW, const V4<T> &RW, T nx, T ny, T g, T epsilon) {
    T A0, U0, V0, H0, P0, A1, U1, V1, H1, P1;
    calc_function(LW, g, A0, U0, V0, H0, P0);
    calc_function(RW, g, A1, U1, V1, H1, P1);
    T M0 = (U0 * nx + V0 * ny);
    T M1 = (U1 * nx + V1 * ny);
    T DVC = M1 - M0;
    T lrou = LW.x, rrou = RW.x;
    T sl = tsqrt(lrou), sr = tsqrt(rrou);
    T ROUB = sl * sr;
    T UB = (U0 * sl + U1 * sr) / (sl + sr);
    T VB = (V0 * sl + V1 * sr) / (sl + sr);
    T HB = (H0 * sl + H1 * sr) / (sl + sr);
    T QB = UB * UB + VB * VB;
    T AB = tsqrt((g - T(1.0)) * (HB - QB / T(2.0)));
    T VC = UB * nx + VB * ny;
    T AD0, AD1, AD2;
    if (tabs(VC - AB) < epsilon) AD0 = ((VC - AB) * (VC - AB) + epsilon * epsilon) / (T(2) * epsilon);
    else AD0 = tabs(VC - AB);
    if (tabs(VC) < epsilon) AD1 = (VC * VC + epsilon * epsilon) / (T(2) * epsilon);
    else AD1 = tabs(VC);
    if (tabs(VC + AB) < epsilon) AD2 = ((VC + AB) * (VC + AB) + epsilon * epsilon) / (T(2) * epsilon);
    else AD2 = tabs(VC + AB);
    T dP = P1 - P0;
    T F00 = AD0 * (dP - ROUB * AB * DVC) / (T(2.0) * AB * AB);
    T F01 = F00 * (UB - AB * nx);
    T F02 = F00 * (VB - AB * ny);
    T F03 = F00 * (HB - AB * VC);
    T F10 = AD1 * ((rrou - lrou) - dP / (AB * AB));
    T F11 = F10 * UB + AD1 * ROUB * (U1 - U0 - DVC * nx);
    T F12 = F10 * VB + AD1 * ROUB * (V1 - V0 - DVC * ny);
    T F13 = F10 * QB * T(0.5) + AD1 * ROUB * (UB * (U1 - U0) + VB * (V1 - V0) - DVC * VC);
    T F20 = AD2 * (dP + ROUB * AB * DVC) / (T(2.0) * AB * AB);
    T F21 = F20 * (UB + AB * nx);
    T F22 = F20 * (VB + AB * ny);
    T F23 = F20 * (HB + AB * VC);
    T WL0 = lrou * M0;
    T WL1 = U0 * WL0 + nx * P0;
    T WL2 = V0 * WL0 + ny * P0;
    T WL3 = WL0 * H0;
    T WR0 = rrou * M1;
    T WR1 = U1 * WR0 + nx * P1;
    T WR2 = V1 * WR0 + ny * P1;
    T WR3 = WR0 * H1;
    V4<T> F;
    F.x = T(0.5) * ((WL0 + WR0) - (F00 + F10 + F20));
    F.y = T(0.5) * ((WL1 + WR1) - (F01 + F11 + F21));
    F.z = T(0.5) * ((WL2 + WR2) - (F02 + F12 + F22));
    F.w = T(0.5) * ((WL3 + WR3) - (F03 + F13 + F23));
    return F;
}

// FP32: the same flux, algebraically identical, arranged for the FP32 units
// (shared reciprocals, explicit fused multiply-adds); the FP32 pass is issue
// bound, not memory bound.  Rounding differs from the generic form at FP32
// level only.
template <>
__device__ __forceinline__ V4<float> roe<float>(const V4<float> &LW, const V4<float> &RW, float nx, float ny,
                                               float g, float epsilon) {
    const float gm1 = g - 1.0f;
    // The left / right quantities as pairs on the packed FP32 units (two
    // lanes per instruction, each with the scalar form's operation order, so
    // the bits are those of the scalar expressions); one reciprocal square
    // root per density gives both its square root and its reciprocal.
    const float2 rho = make_float2(LW.x, RW.x), en = make_float2(LW.w, RW.w);
    const float2 rs = make_float2(frsqrt(LW.x), frsqrt(RW.x));
    const float2 iv = __fmul2_rn(rs, rs);
    const float2 Up = __fmul2_rn(make_float2(LW.y, RW.y), iv), Vp = __fmul2_rn(make_float2(LW.z, RW.z), iv);
    const float2 Pp = __fmul2_rn(make_float2(gm1, gm1),
                                 __ffma2_rn(__fmul2_rn(make_float2(-0.5f, -0.5f), rho),
                                            __ffma2_rn(Up, Up, __fmul2_rn(Vp, Vp)), en));
    const float2 Hp = __fmul2_rn(__fadd2_rn(en, Pp), iv);
    const float2 nx2 = make_float2(nx, nx), ny2 = make_float2(ny, ny);
    const float2 Mp = __ffma2_rn(Up, nx2, __fmul2_rn(Vp, ny2));
    const float2 sp = __fmul2_rn(rho, rs);
    const float U0 = Up.x, U1 = Up.y, V0 = Vp.x, V1 = Vp.y, P0 = Pp.x, P1 = Pp.y, H0 = Hp.x, H1 = Hp.y;
    const float M0 = Mp.x, M1 = Mp.y;
    const float DVC = M1 - M0;
    const float sl = sp.x, sr = sp.y;
    const float ROUB = sl * sr, is = frcp(sl + sr);
    const float UB = fmaf(U0, sl, U1 * sr) * is;
    const float VB = fmaf(V0, sl, V1 * sr) * is;
    const float HB = fmaf(H0, sl, H1 * sr) * is;
    const float QB = fmaf(UB, UB, VB * VB);
    // c^2 of the Roe average: AB = sqrt(c^2) and 1 / AB^2 from one rsqrt
    const float c2 = gm1 * fmaf(-0.5f, QB, HB), rc = frsqrt(c2);
    const float AB = c2 * rc;
    const float VC = fmaf(UB, nx, VB * ny);
    const float e2 = epsilon * epsilon, ie = 0.5f / epsilon;
    // the two acoustic waves (eigenvalues VC -+ AB) as a pair
    const float2 abs2 = make_float2(-AB, AB);
    const float2 lp = __fadd2_rn(make_float2(VC, VC), abs2);  // (VC - AB, VC + AB)
    const float2 lh = __fmul2_rn(__ffma2_rn(lp, lp, make_float2(e2, e2)), make_float2(ie, ie));
    const float AD0 = fabsf(lp.x) < epsilon ? lh.x : fabsf(lp.x);
    const float AD1 = fabsf(VC) < epsilon ? fmaf(VC, VC, e2) * ie : fabsf(VC);
    const float AD2 = fabsf(lp.y) < epsilon ? lh.y : fabsf(lp.y);
    const float dP = P1 - P0, ia2 = rc * rc, rad = ROUB * AB * DVC, h2 = 0.5f * ia2;
    const float2 FA = __fmul2_rn(__fmul2_rn(make_float2(AD0, AD2), __fadd2_rn(make_float2(dP, dP), make_float2(-rad, rad))),
                                 make_float2(h2, h2));  // (F00, F20)
    const float F00 = FA.x, F20 = FA.y;
    const float F10 = AD1 * fmaf(-dP, ia2, RW.x - LW.x);
    const float du = U1 - U0, dv = V1 - V0, aR = AD1 * ROUB;
    const float2 Fk1 = __fmul2_rn(FA, __ffma2_rn(abs2, nx2, make_float2(UB, UB)));  // (F01, F21)
    const float2 Fk2 = __fmul2_rn(FA, __ffma2_rn(abs2, ny2, make_float2(VB, VB)));  // (F02, F22)
    const float2 Fk3 = __fmul2_rn(FA, __ffma2_rn(abs2, make_float2(VC, VC), make_float2(HB, HB)));  // (F03, F23)
    const float F01 = Fk1.x, F21 = Fk1.y, F02 = Fk2.x, F22 = Fk2.y, F03 = Fk3.x, F23 = Fk3.y;
    const float F11 = fmaf(F10, UB, aR * fmaf(-DVC, nx, du));
    const float F12 = fmaf(F10, VB, aR * fmaf(-DVC, ny, dv));
    const float F13 = fmaf(F10 * 0.5f, QB, aR * fmaf(UB, du, fmaf(VB, dv, -DVC * VC)));
    const float2 W0 = __fmul2_rn(rho, Mp);
    const float2 W1 = __ffma2_rn(Up, W0, __fmul2_rn(nx2, Pp));
    const float2 W2 = __ffma2_rn(Vp, W0, __fmul2_rn(ny2, Pp));
    const float2 W3 = __fmul2_rn(W0, Hp);
    const float WL0 = W0.x, WR0 = W0.y, WL1 = W1.x, WR1 = W1.y, WL2 = W2.x, WR2 = W2.y, WL3 = W3.x, WR3 = W3.y;
    V4<float> F;
    F.x = 0.5f * ((WL0 + WR0) - (F00 + F10 + F20));
    F.y = 0.5f * ((WL1 + WR1) - (F01 + F11 + F21));
    F.z = 0.5f * ((WL2 + WR2) - (F02 + F12 + F22));
    F.w = 0.5f * ((WL3 + WR3) - (F03 + F13 + F23));
    return F;
}

// ---------------------------------------------------------------------------
// Pass A: gpu_solver.cu:137-223 (kernel_Boundary), 225-383 (kernel_Gradient),
// 385-454 (kernel_deltT), 456-549 (kernel_Limiter / kernel_LBJinterpolate),
// and the dt part of 768-878 (kernel_Flux_e2c).
// FS[k*n+i] receives the state on the cell's own side of face k: the limited
// reconstruction for an interior face, the cell state itself for a boundary
// face (the reference's boundary faces are first order).
//
// Limiter freezing (an option with no reference counterpart, off when phi is
// null): while not frozen the limiter values of every face are recorded in
// phi; once frozen they are reused instead of re-evaluated, which makes the
// residual a smooth function of the state so that it can converge below the
// limiter's chatter floor.
// Face midpoint minus cell centroid of face k.  FP64 reads the value the host
// computed with the reference's formulas (midpoint and centroid averages,
// gpu_init.cu:100-228), which keeps the FP64 parity bit for bit.  FP32
// derives it from the face vectors already in registers instead of reading 24
// bytes per cell: with e_j = (-S_j.y, S_j.x) the edge opposite node j,
// mid_k - centroid = (e_{k+2} - e_{k+1}) / 6 exactly.
template <typename T>
__device__ __forceinline__ V2<T> face_offset(const MeshDev<T> &m, const V2<T> *S, int k, int i) {
    return m.R[k * m.n + i];
}
template <>
__device__ __forceinline__ V2<float> face_offset<float>(const MeshDev<float> &m, const V2<float> *S, int k, int i) {
    const V2<float> a = S[(k + 1) % 3], b = S[(k + 2) % 3];
    V2<float> r;
    r.x = (a.y - b.y) * (1.0f / 6.0f);
    r.y = (b.x - a.x) * (1.0f / 6.0f);
    return r;
}

// Cell area: FP64 reads the host value (Calc_area, gpu_init.cu:95-98); FP32
// takes half the cross product of two edge vectors, (S_1.x S_2.y - S_1.y S_2.x) / 2
// with the edges e_j = (-S_j.y, S_j.x) of a counter-clockwise cell.
template <typename T>
__device__ __forceinline__ T cell_area(const MeshDev<T> &m, const V2<T> *S, int i) {
    return m.area[i];
}
template <>
__device__ __forceinline__ float cell_area<float>(const MeshDev<float> &m, const V2<float> *S, int i) {
    return 0.5f * fmaf(S[1].x, S[2].y, -(S[1].y * S[2].x));
}

// Limiter value of one component on one face side from its reconstruction
// difference delt2: kind 0 the reference's min(1, (Umax - U) / delt2) for
// delt2 > 0, min(1, (Umin - U) / delt2) for delt2 < 0, 1 for delt2 == 0
// (gpu_solver.cu:456-494; the bound is selected first so a warp divides once
// whatever the signs of its lanes, and a NaN delt2 makes the face state NaN
// whatever the value); kind 1 the Venkatakrishnan form on the same
// differences (option).
template <typename T>
__device__ __forceinline__ T face_limiter(const int kind, const Flow<T> &f, const T A, const T umax, const T umin,
                                          const T u, const T delt2) {
    if (kind == 1) {
        const T e2 = f.venk_k3 * A * tsqrt(A);
        const T d1 = delt2 > T(0) ? umax - u : umin - u;
        return delt2 == T(0) ? T(1.0)
                             : fdiv(d1 * d1 + e2 + T(2) * delt2 * d1, d1 * d1 + T(2) * delt2 * delt2 + d1 * delt2 + e2);
    }
    const T bound = delt2 > T(0) ? umax : umin;
    return delt2 == T(0) ? T(1.0) : tmin(fdiv(bound - u, delt2), T(1.0));
}

// Returns the cell's local time step (also stored in dt[i]).  OPT compiles in
// the scheme options (smooth limiter, frozen limiter values, first-order
// faces, positivity fallback); without them the reference configuration runs
// in fewer registers (no spills at the FP32 occupancy target) with the same
// arithmetic.  first: this iteration uses first-order faces (option).
// FP32, reference configuration: the arithmetic of faces_cell with the
// component pairs (rho, rho u) and (rho v, rho E) on the packed FP32 units
// (two lanes per instruction, each with the scalar operation order, so the
// bits are those of the scalar form): the gradient sums, the gradients, the
// reconstruction differences, the limiter quotients and the face states.
__device__ __forceinline__ float faces_cell_ref32(const MeshDev<float> &m, const Flow<float> &f, const int i,
                                                  const V4<float> *__restrict__ W, V4<float> *__restrict__ FS,
                                                  float *__restrict__ dt) {
    const int n = m.n;
    const int4 tp = m.topo[i];
    const int code[3] = {tp.x, tp.y, tp.z};
    const V4<float> U = W[i];
    V2<float> S[3];
#pragma unroll
    for (int k = 0; k < 3; k++) S[k] = m.S[k * n + i];
    V4<float> nbv[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        nbv[k] = code[k] >= 0 ? W[code[k] >> 3] : ghost(code[k], U, S[k].x, S[k].y, f);
    const float2 U01 = make_float2(U.x, U.y), U23 = make_float2(U.z, U.w), half = make_float2(0.5f, 0.5f);
    float2 g0a = make_float2(0.f, 0.f), g0b = g0a, g1a = g0a, g1b = g0a;
    float jmax[4], jmin[4];
    float Tsum = 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float c = comp(nbv[k], q);
            if (k == 0) { jmax[q] = c; jmin[q] = c; }
            else {
                if (c < jmin[q]) jmin[q] = c;
                if (c > jmax[q]) jmax[q] = c;
            }
        }
        const float2 ha = __fmul2_rn(half, __fadd2_rn(U01, make_float2(nbv[k].x, nbv[k].y)));
        const float2 hb = __fmul2_rn(half, __fadd2_rn(U23, make_float2(nbv[k].z, nbv[k].w)));
        const float2 sx = make_float2(S[k].x, S[k].x), sy = make_float2(S[k].y, S[k].y);
        g0a = __ffma2_rn(ha, sx, g0a);
        g0b = __ffma2_rn(hb, sx, g0b);
        g1a = __ffma2_rn(ha, sy, g1a);
        g1b = __ffma2_rn(hb, sy, g1b);
        Tsum += spectral_radius(U, nbv[k], S[k].y, S[k].x, f.gamma);
    }
    const float A = cell_area(m, S, i);
    const float rA = fdiv(1.0f, A);
    const float2 rA2 = make_float2(rA, rA);
    const float2 gxa = __fmul2_rn(g0a, rA2), gxb = __fmul2_rn(g0b, rA2);
    const float2 gya = __fmul2_rn(g1a, rA2), gyb = __fmul2_rn(g1b, rA2);
    float umax[4], umin[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        umax[q] = tmax(comp(U, q), jmax[q]);
        umin[q] = tmin(comp(U, q), jmin[q]);
    }
    const float2 mone = make_float2(-1.0f, -1.0f);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        V4<float> o = U;
        if (code[k] >= 0) {
            const V2<float> r = face_offset(m, S, k, i);
            const float2 rx = make_float2(r.x, r.x), ry = make_float2(r.y, r.y);
            const float2 da = __ffma2_rn(gxa, rx, __fmul2_rn(gya, ry));  // delt2 of components 0, 1
            const float2 db = __ffma2_rn(gxb, rx, __fmul2_rn(gyb, ry));  // and 2, 3
            // limiter (kind 0): min(1, (bound - u) / delt2), bound - u as
            // u * (-1) + bound (one rounding, the same bits)
            const float2 na = __ffma2_rn(U01, mone, make_float2(da.x > 0.f ? umax[0] : umin[0],
                                                                  da.y > 0.f ? umax[1] : umin[1]));
            const float2 nb = __ffma2_rn(U23, mone, make_float2(db.x > 0.f ? umax[2] : umin[2],
                                                                  db.y > 0.f ? umax[3] : umin[3]));
            const float2 qa = __fmul2_rn(na, make_float2(frcp(da.x), frcp(da.y)));
            const float2 qb = __fmul2_rn(nb, make_float2(frcp(db.x), frcp(db.y)));
            const float2 fa = make_float2(da.x == 0.f ? 1.0f : tmin(qa.x, 1.0f), da.y == 0.f ? 1.0f : tmin(qa.y, 1.0f));
            const float2 fb = make_float2(db.x == 0.f ? 1.0f : tmin(qb.x, 1.0f), db.y == 0.f ? 1.0f : tmin(qb.y, 1.0f));
            const float2 wa = __ffma2_rn(da, fa, U01), wb = __ffma2_rn(db, fb, U23);
            o.x = wa.x; o.y = wa.y; o.z = wb.x; o.w = wb.y;
        }
        FS[k * n + i] = o;
    }
    const float dti = tmin(fdiv(A * f.cfl, Tsum), f.dt_cap);
    dt[i] = dti;
    return dti;
}

// |x| < |y| on the bit patterns (finite values order like their magnitudes'
// bits; a NaN compares above every finite value)
__device__ __forceinline__ bool abs_less(double x, double y) {
    return (unsigned long long)(__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL) <
           (unsigned long long)(__double_as_longlong(y) & 0x7FFFFFFFFFFFFFFFLL);
}

// SRX: the sum of the three face spectral radii comes in as tsum_ext
// (faces_tile evaluates each interior face's radius once per tile).
// LDQ (FP64, reference configuration, called by every lane of the warp; live
// false for padding lanes, which store nothing): the limiter divisions are
// shared out over the warp.  min(1, (bound - u) / delt2) is 1 exactly when
// |bound - u| >= |delt2| (the two have the same sign, and a correctly rounded
// quotient of magnitude >= 1 is >= 1), so only the other slots divide: each
// lane parks those (numerator, delt2) pairs in its row of qv (12 slots x 2),
// the warp lists them in qi, every lane divides list entries lane, lane + 32,
// ..., and reads its quotients back.  Same operands, same IEEE division: the
// bits do not change; a warp divides about 2-3 times per lane instead of 12.
template <typename T, bool OPT, bool SRX = false, bool LDQ = false>
__device__ __forceinline__ T faces_cell(const MeshDev<T> &m, const Flow<T> &f, const int i,
                                        const V4<T> *__restrict__ W, V4<T> *__restrict__ FS,
                                        T *__restrict__ dt, V4<T> *__restrict__ phi, const int frozen,
                                        const bool first = false, const T tsum_ext = T(0),
                                        T *qv_warp = nullptr, unsigned short *qi = nullptr, const bool live = true) {
    if constexpr (sizeof(T) == 4 && !OPT && !SRX && !LDQ) return faces_cell_ref32(m, f, i, W, FS, dt);
    const int n = m.n;
    const int4 tp = m.topo[i];
    const int code[3] = {tp.x, tp.y, tp.z};
    const V4<T> U = W[i];
    V2<T> S[3];
#pragma unroll
    for (int k = 0; k < 3; k++) S[k] = m.S[k * n + i];
    V4<T> nbv[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        nbv[k] = code[k] >= 0 ? W[code[k] >> 3] : ghost(code[k], U, S[k].x, S[k].y, f);
    T g0[4] = {T(0.0), T(0.0), T(0.0), T(0.0)}, g1[4] = {T(0.0), T(0.0), T(0.0), T(0.0)};
    T jmax[4], jmin[4];
    T Tsum = T(0);
#pragma unroll
    for (int k = 0; k < 3; k++) {
#pragma unroll
        for (int q = 0; q < 4; q++) {
            T c = comp(nbv[k], q);
            if (k == 0) { jmax[q] = c; jmin[q] = c; }
            else {
                if (c < jmin[q]) jmin[q] = c;
                if (c > jmax[q]) jmax[q] = c;
            }
            T u = comp(U, q);
            g0[q] = madd(T(0.5) * (u + c), S[k].x, g0[q]);
            g1[q] = madd(T(0.5) * (u + c), S[k].y, g1[q]);
        }
        if (!SRX) Tsum += spectral_radius(U, nbv[k], S[k].y, S[k].x, f.gamma);
    }
    if (SRX) Tsum = tsum_ext;
    const T A = cell_area(m, S, i);
    const T rA = fdiv(T(1.0), A);
    T gx[4], gy[4], umax[4], umin[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        gx[q] = g0[q] * rA;
        gy[q] = g1[q] * rA;
        umax[q] = tmax(comp(U, q), jmax[q]);
        umin[q] = tmin(comp(U, q), jmin[q]);
    }
    const bool reuse = OPT && phi && frozen;
    // cell-wise limiter options (2, 3): the smallest of the per-face values of
    // the cell's interior faces (reference form, Venkatakrishnan form), the
    // same value on every face of the cell
    const bool cellwise = OPT && f.limiter >= 2;
    T phic[4] = {T(1.0), T(1.0), T(1.0), T(1.0)};
    if (cellwise && !reuse && !first) {
#pragma unroll
        for (int q = 0; q < 4; q++) phic[q] = T(INFINITY);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (code[k] < 0) continue;
            const V2<T> r = face_offset(m, S, k, i);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const T delt2 = madd(gx[q], r.x, gy[q] * r.y);
                phic[q] = tmin(phic[q], face_limiter(f.limiter - 2, f, A, umax[q], umin[q], comp(U, q), delt2));
            }
        }
    }
    unsigned need = 0;
    T *qv = nullptr;
    if constexpr (LDQ) {
        const int lane = threadIdx.x & 31;
        qv = qv_warp + lane * 24;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (code[k] < 0) continue;
            const V2<T> r = face_offset(m, S, k, i);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int sl = 4 * k + q;
                const T delt2 = madd(gx[q], r.x, gy[q] * r.y);
                const T num = (delt2 > T(0) ? umax[q] : umin[q]) - comp(U, q);
                if (live && delt2 != T(0) && abs_less(num, delt2)) {
                    need |= 1u << sl;
                    qv[2 * sl] = num;
                    qv[2 * sl + 1] = delt2;
                }
            }
        }
        const int cnt = __popc(need);
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        int off = incl - cnt;
        for (unsigned mm = need; mm; mm &= mm - 1) qi[off++] = (unsigned short)((lane << 4) | (__ffs(mm) - 1));
        __syncwarp();
        for (int j = lane; j < total; j += 32) {
            const int e = qi[j];
            T *pv = qv_warp + (e >> 4) * 24 + 2 * (e & 15);
            pv[0] = pv[0] / pv[1];
        }
        __syncwarp();
        if (!live) return T(0);
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        V4<T> o = U;
        if (code[k] >= 0 && !(OPT && first)) {
            const V2<T> r = face_offset(m, S, k, i);
            V4<T> pf;
            if (reuse) pf = phi[k * n + i];
            T fi = T(1.0), d[4], ph[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                T delt2 = madd(gx[q], r.x, gy[q] * r.y);
                T u = comp(U, q);
                if (reuse) fi = comp(pf, q);
                else if (cellwise) fi = phic[q];
                else if (LDQ) fi = (need >> (4 * k + q)) & 1 ? tmin(qv[2 * (4 * k + q)], T(1.0)) : T(1.0);
                else fi = face_limiter(OPT ? f.limiter : 0, f, A, umax[q], umin[q], u, delt2);
                ph[q] = fi;
                d[q] = madd(delt2, fi, u);
            }
            o.x = d[0]; o.y = d[1]; o.z = d[2]; o.w = d[3];
            if (OPT && f.positivity) {
                // positivity fallback (option): a face side with a density or
                // pressure that is not positive takes the cell state
                const T q = T(0.5) * (d[1] * d[1] + d[2] * d[2]) / d[0];
                if (!(d[0] > T(0)) || !((f.gamma - T(1.0)) * (d[3] - q) > T(0))) o = U;
            }
            if (OPT && phi && !frozen) {
                V4<T> pw;
                pw.x = ph[0]; pw.y = ph[1]; pw.z = ph[2]; pw.w = ph[3];
                phi[k * n + i] = pw;
            }
        }
        FS[k * n + i] = o;
    }
    const T dti = tmin(fdiv(A * f.cfl, Tsum), f.dt_cap);
    dt[i] = dti;
    return dti;
}

// Pass A for one tile of cells [base, base + nvalid) with each interior
// face's spectral radius evaluated once (the FP64 path, bound by the FP64
// rate: the radius takes 4 divisions and a square root): the tile lists the
// radii it must evaluate (boundary faces, faces to cells outside the tile,
// and inside faces from their left cell only, as flux_tile does for the Roe
// flux), spreads that list over its threads with the cell states in shared
// memory, then every cell sums its three radii in face order and runs the
// rest of faces_cell.  The radius is symmetric in its two states and in the
// sign of the face vector, and the two cells of a face hold exactly negated
// face vectors, so each cell gets the bits of its own evaluation.
// The limiter divisions are shared out over each warp (faces_cell, LDQ).
// blockDim.x <= kFacesTile.
constexpr int kFacesTile = 128;
template <typename T>
__device__ __forceinline__ void faces_tile(const MeshDev<T> &m, const Flow<T> &f, const int base, const int nvalid,
                                           const V4<T> *__restrict__ W, V4<T> *__restrict__ FS,
                                           T *__restrict__ dt) {
    __shared__ V4<T> Us[kFacesTile];
    __shared__ int4 tps[kFacesTile];
    __shared__ T SRs[kFacesTile * 3];
    __shared__ unsigned short items[kFacesTile * 3];
    __shared__ int wtot[kFacesTile / 32];
    __shared__ T qv[kFacesTile * 24];
    __shared__ unsigned short qi[kFacesTile * 12];
    const int n = m.n, t = threadIdx.x, i = base + t;
    const bool live = t < nvalid;
    const int4 tp = live ? m.topo[i] : make_int4(-3, -3, -3, 0);
    tps[t] = tp;
    if (live) Us[t] = W[i];
    const int code[3] = {tp.x, tp.y, tp.z};
    unsigned mask = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (!live) continue;
        const int c = code[k];
        if (c < 0) { mask |= 1u << k; continue; }
        const bool inside = (unsigned)((c >> 3) - base) < (unsigned)nvalid;
        if (!inside || !((c >> 2) & 1)) mask |= 1u << k;
    }
    // exclusive prefix sum of the per-cell counts over the block
    const int cnt = __popc(mask), lane = t & 31, wid = t >> 5;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wtot[wid] = incl;
    __syncthreads();
    int off = incl - cnt, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        if (w < wid) off += wtot[w];
        total += wtot[w];
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
        if (mask & (1u << k)) items[off++] = (unsigned short)((t << 2) | k);
    __syncthreads();
    for (int j = t; j < total; j += blockDim.x) {
        const int it = items[j], tt = it >> 2, k = it & 3;
        const int4 q = tps[tt];
        const int c = k == 0 ? q.x : k == 1 ? q.y : q.z;
        const V4<T> Uo = Us[tt];
        const V2<T> S = m.S[k * n + base + tt];
        V4<T> nb;
        if (c >= 0) {
            const int nj = c >> 3;
            nb = (unsigned)(nj - base) < (unsigned)nvalid ? Us[nj - base] : W[nj];
        } else {
            nb = ghost(c, Uo, S.x, S.y, f);
        }
        SRs[tt * 3 + k] = spectral_radius(Uo, nb, S.y, S.x, f.gamma);
    }
    __syncthreads();
    T Tsum = T(1);
    if (live) {
        Tsum = T(0);
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const int c = code[k];
            Tsum += (mask & (1u << k)) ? SRs[t * 3 + k] : SRs[((c >> 3) - base) * 3 + (c & 3)];
        }
    }
    // every lane of a warp takes part in the shared limiter divisions; a
    // padding lane computes on the tile's first cell and stores nothing
    const int w = t >> 5;
    faces_cell<T, false, true, true>(m, f, live ? i : base, W, FS, dt, nullptr, 0, false, Tsum, qv + w * 32 * 24,
                                     qi + w * 32 * 12, live);
}

// Pass A of the reference configuration in tiles (FP64, see faces_tile).
template <typename T>
__global__ void E2D_LB_FACES k_faces_tile(MeshDev<T> m, Flow<T> f, const V4<T> *__restrict__ W,
                                          V4<T> *__restrict__ FS, T *__restrict__ dt, Ctl *__restrict__ ctl,
                                          V4<T> *__restrict__ phi, const int st) {
    wait_prior_grid();
    if (ctl->halt) return;
    const int base = blockIdx.x * blockDim.x;
    faces_tile(m, f, base, min((int)blockDim.x, m.n - base), W, FS, dt);
}
template <typename T> struct FacesTiled { static constexpr bool value = sizeof(T) == 8; };
template <typename T> inline bool faces_tiled(int block) { return FacesTiled<T>::value && block <= kFacesTile; }

// Global time-step option: the block's smallest step folded into *slot.
// Every thread of the block must call it (v = +inf for no cell).  A time
// step is non-negative, so its bits order like the integers and min over
// them is exact and independent of the order of the blocks.
__device__ __forceinline__ void block_min_dt(double v, unsigned long long *slot) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    __shared__ double wm[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // wm may still be read by the previous use in this block
    if (lane == 0) wm[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = wm[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); k++) b = fmin(b, wm[k]);
        atomicMin(slot, (unsigned long long)__double_as_longlong(b));
    }
}

// OPT: the variant with the scheme options (smooth limiter, limiter freezing,
// global time step); faces_options picks it.
template <typename T, bool OPT>
__global__ void E2D_LB_FACES k_faces(MeshDev<T> m, Flow<T> f, const V4<T> *__restrict__ W,
                                     V4<T> *__restrict__ FS, T *__restrict__ dt,
                                     Ctl *__restrict__ ctl, V4<T> *__restrict__ phi, const int st) {
    wait_prior_grid();
    if (ctl->halt) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool first = OPT && ctl->step < f.first_order;
    if (!OPT || !f.global_dt) {
        if (i >= m.n) return;
        faces_cell<T, OPT>(m, f, i, W, FS, dt, phi, OPT && phi ? ctl->frozen : 0, first);
        return;
    }
    double v = __longlong_as_double((long long)kDtNone);
    if (i < m.n) v = (double)faces_cell<T, OPT>(m, f, i, W, FS, dt, phi, phi ? ctl->frozen : 0, first);
    block_min_dt(v, &ctl->dtmin[st]);
}

// True when a pass-A launch needs the option variant.
template <typename T> inline bool faces_options(const Flow<T> &f, const void *phi) {
    return phi != nullptr || f.limiter != 0 || f.global_dt != 0 || f.first_order > 0 || f.positivity != 0;
}

// Time step of cell i in RK stage st: its own, or with the global option the
// smallest of its case.
template <typename T>
__device__ __forceinline__ T stage_dt(const Flow<T> &f, const Ctl *ctl, const int st, const T *dt, const int i) {
    return f.global_dt ? (T)__longlong_as_double((long long)ctl->dtmin[st]) : dt[i];
}

// ---------------------------------------------------------------------------
// Pass B: gpu_solver.cu:651-764 (kernel_Flux2) evaluated per cell for its
// three faces, summed as gpu_solver.cu:798-825 (+F where the cell is the
// edge's left cell, -F where it is the right cell, in face order).
template <typename T>
__device__ __forceinline__ void flux_cell(const MeshDev<T> &m, const Flow<T> &f, const int i,
                                          const V4<T> *__restrict__ FS, V4<T> *__restrict__ res) {
    const int n = m.n;
    const int4 tp = m.topo[i];
    const int code[3] = {tp.x, tp.y, tp.z};
    V4<T> r;
    r.x = T(0.0); r.y = T(0.0); r.z = T(0.0); r.w = T(0.0);
    // every input of the three faces is requested before the first flux
    V2<T> S[3];
    V4<T> own[3], oth[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        S[k] = m.S[k * n + i];
        own[k] = FS[k * n + i];
        if (code[k] >= 0) oth[k] = FS[(code[k] & 3) * n + (code[k] >> 3)];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        bool right;
        const V4<T> F = face_flux_of(f, code[k], S[k], own[k], oth[k], right);
        if constexpr (sizeof(T) == 4) {
            // r +- F as r + (+-1) F: the product is exact, one rounding, the
            // same bits as the add or subtract; two packed instructions
            const float sg = right ? -1.0f : 1.0f;
            const float2 xy = __ffma2_rn(make_float2(F.x, F.y), make_float2(sg, sg), make_float2(r.x, r.y));
            const float2 zw = __ffma2_rn(make_float2(F.z, F.w), make_float2(sg, sg), make_float2(r.z, r.w));
            r.x = xy.x; r.y = xy.y; r.z = zw.x; r.w = zw.y;
        } else {
            if (right) { r.x -= F.x; r.y -= F.y; r.z -= F.z; r.w -= F.w; }
            else { r.x += F.x; r.y += F.y; r.z += F.z; r.w += F.w; }
        }
    }
    res[i] = r;
}

// Length vn of the face vector S and the unit normal S / vn: IEEE in FP64; in
// FP32 from one reciprocal square root of |S|^2 (the other cell of the face,
// with S negated, gets the exact negative).
template <typename T> __device__ __forceinline__ void unit_normal(const V2<T> S, T &nx, T &ny, T &vn) {
    vn = tsqrt(S.y * S.y + S.x * S.x);
    nx = S.x / vn;
    ny = S.y / vn;
}
template <> __device__ __forceinline__ void unit_normal<float>(const V2<float> S, float &nx, float &ny, float &vn) {
    const float q = fmaf(S.y, S.y, S.x * S.x), r = frsqrt(q);
    vn = q * r;
    const float2 nn = __fmul2_rn(make_float2(S.x, S.y), make_float2(r, r));
    nx = nn.x;
    ny = nn.y;
}

// Inputs of the Roe flux of one face in the edge's orientation: left state a,
// right state b (the ghost across a boundary face), unit normal (nx, ny) of
// the edge and the face length vn; *right tells whether the cell is the
// edge's right cell.
template <typename T>
__device__ __forceinline__ void face_inputs(const Flow<T> &f, const int code, const V2<T> S, const V4<T> own,
                                            const V4<T> oth, V4<T> &a, V4<T> &b, T &nx, T &ny, T &vn,
                                            bool &right) {
    unit_normal(S, nx, ny, vn);
    // the left state first: both cells of a face run the same instructions on
    // the same inputs (their normals are exact negatives), so they get the
    // same bits
    a = own;
    right = false;
    if (code >= 0) {
        right = (code >> 2) & 1;
        if (right) { a = oth; b = own; nx = -nx; ny = -ny; }
        else b = oth;
    } else {
        b = ghost(code, own, S.x, S.y, f);
    }
}

// Flux of face k of cell i, times |S|, in the edge's orientation (the
// reference's Res_e.left of gpu_solver.cu:738-745); *right tells whether cell
// i is the edge's right cell.
template <typename T>
__device__ __forceinline__ V4<T> face_flux_of(const Flow<T> &f, const int code, const V2<T> S, const V4<T> own,
                                              const V4<T> oth, bool &right) {
    V4<T> a, b;
    T nx, ny, vn;
    face_inputs(f, code, S, own, oth, a, b, nx, ny, vn, right);
    // one Roe call site for every face
    V4<T> F = roe(a, b, nx, ny, f.gamma, f.eps_entropy);
    if constexpr (sizeof(T) == 4) {
        // two packed multiplies, the same products
        const float2 xy = __fmul2_rn(make_float2(F.x, F.y), make_float2(vn, vn));
        const float2 zw = __fmul2_rn(make_float2(F.z, F.w), make_float2(vn, vn));
        F.x = xy.x; F.y = xy.y; F.z = zw.x; F.w = zw.y;
    } else {
        F.x *= vn; F.y *= vn; F.z *= vn; F.w *= vn;
    }
    return F;
}

template <typename T>
__device__ __forceinline__ V4<T> face_flux(const MeshDev<T> &m, const Flow<T> &f, const int i, const int k,
                                           const int code, const V4<T> *__restrict__ FS, bool &right) {
    const int n = m.n;
    const V2<T> S = m.S[k * n + i];
    const V4<T> own = FS[k * n + i];
    V4<T> oth = own;
    if (code >= 0) oth = FS[(code & 3) * n + (code >> 3)];
    return face_flux_of(f, code, S, own, oth, right);
}

// Pass B for one tile of cells [base, base + nvalid) with each interior face
// inside the tile evaluated once: the tile lists the faces it must evaluate
// (boundary faces, faces to cells outside the tile, and inside faces from
// their left cell only), spreads that list over its threads, keeps the
// fluxes in shared memory, and then every cell sums its three faces in face
// order with the reference's signs.  The fluxes are the same bits as in
// flux_cell and are summed in the same order.  blockDim.x <= 256.
template <typename T>
__device__ __forceinline__ void flux_tile(const MeshDev<T> &m, const Flow<T> &f, const int base, const int nvalid,
                                          const V4<T> *__restrict__ FS, V4<T> *__restrict__ res) {
    __shared__ V4<T> Fs[256 * 3];
    __shared__ int4 tps[256];
    __shared__ unsigned short items[256 * 3];
    __shared__ int wtot[8];
    const int t = threadIdx.x, i = base + t;
    const bool live = t < nvalid;
    const int4 tp = live ? m.topo[i] : make_int4(-3, -3, -3, 0);
    tps[t] = tp;
    const int code[3] = {tp.x, tp.y, tp.z};
    unsigned mask = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (!live) continue;
        const int c = code[k];
        if (c < 0) { mask |= 1u << k; continue; }
        const bool inside = (unsigned)((c >> 3) - base) < (unsigned)nvalid;
        if (!inside || !((c >> 2) & 1)) mask |= 1u << k;
    }
    // exclusive prefix sum of the per-cell counts over the block
    const int cnt = __popc(mask), lane = t & 31, wid = t >> 5;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wtot[wid] = incl;
    __syncthreads();
    int off = incl - cnt, total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
        if (w < wid) off += wtot[w];
        total += wtot[w];
    }
#pragma unroll
    for (int k = 0; k < 3; k++)
        if (mask & (1u << k)) items[off++] = (unsigned short)((t << 2) | k);
    __syncthreads();
    for (int j = t; j < total; j += blockDim.x) {
        const int it = items[j], tt = it >> 2, k = it & 3;
        const int4 q = tps[tt];
        const int c = k == 0 ? q.x : k == 1 ? q.y : q.z;
        bool right;
        Fs[tt * 3 + k] = face_flux(m, f, base + tt, k, c, FS, right);
    }
    __syncthreads();
    if (!live) return;
    V4<T> r;
    r.x = T(0.0); r.y = T(0.0); r.z = T(0.0); r.w = T(0.0);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const int c = code[k];
        V4<T> F;
        bool right;
        if (mask & (1u << k)) {
            F = Fs[t * 3 + k];
            right = c >= 0 && ((c >> 2) & 1);
        } else {  // inside face evaluated by its left cell
            F = Fs[((c >> 3) - base) * 3 + (c & 3)];
            right = true;
        }
        if (right) { r.x -= F.x; r.y -= F.y; r.z -= F.z; r.w -= F.w; }
        else { r.x += F.x; r.y += F.y; r.z += F.z; r.w += F.w; }
    }
    res[i] = r;
}

template <typename T>
__global__ void E2D_LB_FLUX k_flux_tile(MeshDev<T> m, Flow<T> f, const V4<T> *__restrict__ FS,
                                        V4<T> *__restrict__ res, const Ctl *__restrict__ ctl) {
    wait_prior_grid();
    if (ctl->halt) return;
    const int base = blockIdx.x * blockDim.x;
    flux_tile(m, f, base, min((int)blockDim.x, m.n - base), FS, res);
}

template <typename T>
__global__ void E2D_LB_FLUX k_flux(MeshDev<T> m, Flow<T> f, const V4<T> *__restrict__ FS,
                                   V4<T> *__restrict__ res, const Ctl *__restrict__ ctl) {
    wait_prior_grid();
    if (ctl->halt) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n) return;
    flux_cell(m, f, i, FS, res);
}

// Sum of the interior neighbours' values in face order (gpu_solver.cu:1658-1666)
template <typename T>
__device__ __forceinline__ V4<T> nb_sum(const int4 tp, const V4<T> *__restrict__ src) {
    V4<T> d;
    d.x = T(0.0); d.y = T(0.0); d.z = T(0.0); d.w = T(0.0);
    const int code[3] = {tp.x, tp.y, tp.z};
#pragma unroll
    for (int k = 0; k < 3; k++)
        if (code[k] >= 0) {
            const V4<T> v = src[code[k] >> 3];
            d.x += v.x; d.y += v.y; d.z += v.z; d.w += v.w;
        }
    return d;
}

// ---------------------------------------------------------------------------
// Pass C: gpu_solver.cu:1635-1673 (kernel_Smooth1): one Jacobi-type sweep
// dst = (eps * sum_interior src + res) / (1 + eps * CLog).
template <typename T>
__device__ __forceinline__ void smooth_cell(const MeshDev<T> &m, const T eps, const int i,
                                            const V4<T> *__restrict__ src, const V4<T> *__restrict__ res,
                                            V4<T> *__restrict__ dst) {
    const int4 tp = m.topo[i];
    const V4<T> d = nb_sum(tp, src);
    const V4<T> r0 = res[i];
    const T den = T(1.0) + (eps) * T(tp.w);
    V4<T> o;
    o.x = fdiv(madd(d.x, eps, r0.x), den);
    o.y = fdiv(madd(d.y, eps, r0.y), den);
    o.z = fdiv(madd(d.z, eps, r0.z), den);
    o.w = fdiv(madd(d.w, eps, r0.w), den);
    dst[i] = o;
}

template <typename T>
__global__ void __launch_bounds__(256) k_smooth(MeshDev<T> m, T eps, const V4<T> *__restrict__ src,
                                                const V4<T> *__restrict__ res, V4<T> *__restrict__ dst,
                                                const Ctl *__restrict__ ctl) {
    wait_prior_grid();
    if (ctl->halt) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m.n) return;
    smooth_cell(m, eps, i, src, res, dst);
}

// ---------------------------------------------------------------------------
// Pass D: gpu_solver.cu:1675-1720 (kernel_Smooth2, last sweep + clamp) fused
// with 938-966 (kernel_RKStep); on the last stage also 968-1020 (kernel_drou)
// as FP64 block partials and a count of unphysical cells.
template <typename T>
__device__ __forceinline__ void update_cell(const MeshDev<T> &m, const Flow<T> &f, const T rk,
                                            const int smooth, const int i, const V4<T> *__restrict__ src,
                                            const V4<T> *__restrict__ res, const T dti,
                                            const V4<T> *W0, V4<T> *Wout, const bool want, T &drho,
                                            int &bad) {
    {
        const int4 tp = m.topo[i];
        V4<T> r = res[i];
        if (smooth) {
            const V4<T> d = nb_sum(tp, src);
            const T eps = f.irs_eps;
            const T den = T(1.0) + (eps) * T(tp.w);
            T s0 = fdiv(madd(d.x, eps, r.x), den), s1 = fdiv(madd(d.y, eps, r.y), den);
            T s2 = fdiv(madd(d.z, eps, r.z), den), s3 = fdiv(madd(d.w, eps, r.w), den);
            if (tabs(r.x) > tabs(s0)) r.x = s0;
            if (tabs(r.y) > tabs(s1)) r.y = s1;
            if (tabs(r.z) > tabs(s2)) r.z = s2;
            if (tabs(r.w) > tabs(s3)) r.w = s3;
        }
        T RK = rk;
        RK *= dti;
        const T A = m.area[i];
        const V4<T> w0 = W0[i];
        V4<T> w;
        w.x = w0.x - fdiv(RK * r.x, A);
        w.y = w0.y - fdiv(RK * r.y, A);
        w.z = w0.z - fdiv(RK * r.z, A);
        w.w = w0.w - fdiv(RK * r.w, A);
        Wout[i] = w;
        if (want) {
            // rho - rho0 in the stencil's precision: exact in FP32 as long as the
            // two densities are within a factor of two (Sterbenz)
            drho = w.x - w0.x;
            const T q = T(0.5) * (w.y * w.y + w.z * w.z) / w.x;
            bad = !(w.x > T(0)) || !(w.w - q > T(0));
        }
    }
}

// Deterministic block sum of (rho - rho0)^2 (fixed shuffle tree, then the
// warps in order) into *slot, and the count of unphysical cells added to
// *nbad.  Every thread of the block must call it.  FP64 stencil: an FP64 sum.
// FP32 stencil: the squares and sums as unevaluated pairs of floats (exact
// square by a fused multiply-add, two-sum additions), about 48 bits, so that
// pass D issues no FP64 instruction (FP64 throughput is a small fraction of
// FP32 on this GPU and the FP64 tree took ~25 us per iteration at 4.2M
// cells); *slot then holds the pair as a float2 that the residual kernel
// widens to FP64.
__device__ __forceinline__ void block_partial(double drho, int bad, double *slot, int *nbad) {
    double d2 = drho * drho;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d2 += __shfl_down_sync(0xffffffffu, d2, o);
    unsigned badmask = __ballot_sync(0xffffffffu, bad);
    __shared__ double ws[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // ws may still be read by the previous use in this block
    if (lane == 0) {
        ws[wid] = d2;
        if (badmask) atomicAdd(nbad, __popc(badmask));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += ws[k];
        *slot = s;
    }
}

// a + b for unevaluated float pairs (a.x + a.y): two-sum of the leading
// parts, the trailing parts and its error added, renormalised.  The terms
// summed here are non-negative, so there is no cancellation.
__device__ __forceinline__ void pair_add(float &ah, float &al, const float bh, const float bl) {
    const float s = ah + bh;
    const float bb = s - ah;
    const float e = (ah - (s - bb)) + (bh - bb);
    const float t = e + (al + bl);
    ah = s + t;
    al = t - (ah - s);
}

__device__ __forceinline__ void block_partial(float drho, int bad, double *slot, int *nbad) {
    float hi = drho * drho;
    float lo = fmaf(drho, drho, -hi);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float bh = __shfl_down_sync(0xffffffffu, hi, o), bl = __shfl_down_sync(0xffffffffu, lo, o);
        pair_add(hi, lo, bh, bl);
    }
    unsigned badmask = __ballot_sync(0xffffffffu, bad);
    __shared__ float2 wsf[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();  // wsf may still be read by the previous use in this block
    if (lane == 0) {
        wsf[wid] = make_float2(hi, lo);
        if (badmask) atomicAdd(nbad, __popc(badmask));
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float sh = 0.0f, sl = 0.0f;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) pair_add(sh, sl, wsf[k].x, wsf[k].y);
        *reinterpret_cast<float2 *>(slot) = make_float2(sh, sl);
    }
}

// GDT: the global time-step option (its FP64 slot is converted per thread, an
// FP64-pipe instruction the local-step variant does without).
template <typename T, bool GDT>
__global__ void __launch_bounds__(256) k_update(MeshDev<T> m, Flow<T> f, T rk, int smooth,
                                                const V4<T> *__restrict__ src, const V4<T> *__restrict__ res,
                                                const T *__restrict__ dt, const V4<T> *W0, V4<T> *Wout,
                                                double *__restrict__ part, Ctl *ctl, const int st) {
    wait_prior_grid();
    if (ctl->halt) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    T drho = T(0.0);
    int bad = 0;
    if (i < m.n)
        update_cell(m, f, rk, smooth, i, src, res,
                    GDT ? (T)__longlong_as_double((long long)ctl->dtmin[st]) : dt[i], W0, Wout, part != nullptr,
                    drho, bad);
    if (!part) return;
    block_partial(drho, bad, part + blockIdx.x, &ctl->nbad);
}

// ---------------------------------------------------------------------------
// Batched cases: the same per-cell work as the kernels above, by persistent
// CTAs that walk the tiles of all cases (tile = blockDim.x consecutive cells,
// all of one case: cases are padded to kChunk cells and a block has at most
// kChunk threads).  The tile's case, its halt flag and its flow constants are
// looked up once per tile (uniform over the block); tiles of halted
// (converged) cases and padding cells are skipped.

template <typename T, bool OPT>
__global__ void __launch_bounds__(256, BatchMinBlocks<T>::faces) kb_faces(MeshDev<T> m, BatchDev<T> b, int ntiles, const V4<T> *__restrict__ W,
                                      V4<T> *__restrict__ FS, T *__restrict__ dt, V4<T> *__restrict__ phi,
                                      const int st) {
    wait_prior_grid();
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int base = t * blockDim.x, i = base + threadIdx.x;
        const int tc = b.chunk_case[base / kChunk];  // the tile's case
        if (b.ctl[tc].halt) continue;                // uniform over the block
        const Flow<T> f = b.flows[tc];
        double v = __longlong_as_double((long long)kDtNone);
        if (i < b.case_end[tc])
            v = (double)faces_cell<T, OPT>(m, f, i, W, FS, dt, phi, OPT && phi ? b.ctl[tc].frozen : 0,
                                           OPT && b.ctl[tc].step < f.first_order);
        if (OPT && f.global_dt) block_min_dt(v, &b.ctl[tc].dtmin[st]);  // uniform over the block
    }
}

template <typename T>
__global__ void __launch_bounds__(256, BatchMinBlocks<T>::flux) kb_flux(MeshDev<T> m, BatchDev<T> b, int ntiles, const V4<T> *__restrict__ FS,
                                    V4<T> *__restrict__ res) {
    wait_prior_grid();
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int base = t * blockDim.x;
        const int tc = b.chunk_case[base / kChunk];  // every cell of a tile is in one case
        if (b.ctl[tc].halt) continue;                // uniform over the block
        const Flow<T> f = b.flows[tc];
        if constexpr (FluxTiled<T>::value) {
            flux_tile(m, f, base, max(0, min((int)blockDim.x, b.case_end[tc] - base)), FS, res);
        } else {
            const int i = base + threadIdx.x;
            if (i < b.case_end[tc]) flux_cell(m, f, i, FS, res);
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256) kb_smooth(MeshDev<T> m, BatchDev<T> b, int ntiles, T eps,
                                                 const V4<T> *__restrict__ src, const V4<T> *__restrict__ res,
                                                 V4<T> *__restrict__ dst) {
    wait_prior_grid();
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int base = t * blockDim.x, i = base + threadIdx.x;
        const int tc = b.chunk_case[base / kChunk];
        if (b.ctl[tc].halt) continue;
        if (i < b.case_end[tc]) smooth_cell(m, eps, i, src, res, dst);
    }
}

// GDT: some case uses the global time-step option (read per case); without
// it the FP32 build issues no FP64 conversion.
template <typename T, bool GDT>
__global__ void __launch_bounds__(256) kb_update(MeshDev<T> m, BatchDev<T> b, int ntiles, T rk, int smooth,
                                                 const V4<T> *__restrict__ src, const V4<T> *__restrict__ res,
                                                 const T *__restrict__ dt, const V4<T> *W0, V4<T> *Wout,
                                                 double *__restrict__ part, const int st) {
    wait_prior_grid();
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int base = t * blockDim.x, i = base + threadIdx.x;
        const int tc = b.chunk_case[base / kChunk];  // the tile's case
        if (b.ctl[tc].halt) continue;                // uniform over the block
        T drho = T(0.0);
        int bad = 0;
        if (i < b.case_end[tc]) {
            const Flow<T> f = b.flows[tc];
            update_cell(m, f, rk, smooth, i, src, res, GDT ? stage_dt(f, &b.ctl[tc], st, dt, i) : dt[i], W0, Wout,
                        part != nullptr, drho, bad);
        }
        if (part) block_partial(drho, bad, part + t, &b.ctl[tc].nbad);
    }
}

// One iteration of every case that has not halted; the same stage / buffer
// sequence as enqueue_iteration.
template <typename T> void enqueue_batch_iteration(const BPlan<T> &p, cudaStream_t s) {
    const int B = p.block, NT = (p.m.n + B - 1) / B, G = p.grid;
    for (int st = 0; st < p.stages; st++) {
        const bool last = st == p.stages - 1;
        V4<T> *Wcur = st == 0 ? p.W[0] : p.W[1];
        V4<T> *Wout = last ? p.W[0] : p.W[1];
        if (p.options) launch_chained(kb_faces<T, true>, G, B, s, p.m, p.b, NT, Wcur, p.FS, p.dt, p.phi, st);
        else launch_chained(kb_faces<T, false>, G, B, s, p.m, p.b, NT, Wcur, p.FS, p.dt, p.phi, st);
        launch_chained(kb_flux<T>, G, B, s, p.m, p.b, NT, p.FS, p.res);
        const V4<T> *src = p.res;
        for (int sw = 0; sw + 1 < p.sweeps; sw++) {
            V4<T> *dst = p.sm[sw & 1];
            launch_chained(kb_smooth<T>, G, B, s, p.m, p.b, NT, p.f.irs_eps, src, p.res, dst);
            src = dst;
        }
        if (p.options)
            launch_chained(kb_update<T, true>, G, B, s, p.m, p.b, NT, p.rk[st], p.sweeps > 0 ? 1 : 0, src, p.res,
                           p.dt, p.W[0], Wout, last ? p.part : nullptr, st);
        else
            launch_chained(kb_update<T, false>, G, B, s, p.m, p.b, NT, p.rk[st], p.sweeps > 0 ? 1 : 0, src, p.res,
                           p.dt, p.W[0], Wout, last ? p.part : nullptr, st);
    }
    enqueue_batch_resid(p.part, p.case_tiles, p.ncase, p.b.ctl, p.hist, p.hist_cap, sizeof(T) == 4, s);
}

// ---------------------------------------------------------------------------
// State exchange with the caller: FP64 in file order <-> T in internal order.
template <typename T>
__global__ void k_import(int n, const int *__restrict__ perm, const double *__restrict__ wfile,
                         V4<T> *__restrict__ W) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *s = wfile + 4 * (size_t)perm[i];
    V4<T> o;
    o.x = (T)s[0]; o.y = (T)s[1]; o.z = (T)s[2]; o.w = (T)s[3];
    W[i] = o;
}

template <typename T>
__global__ void k_export(int n, const int *__restrict__ perm, const V4<T> *__restrict__ W,
                         double *__restrict__ wfile) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V4<T> v = W[i];
    double *d = wfile + 4 * (size_t)perm[i];
    d[0] = (double)v.x; d[1] = (double)v.y; d[2] = (double)v.z; d[3] = (double)v.w;
}

template <typename T>
void enqueue_import(int n, const int *perm, const double *wfile, V4<T> *W, cudaStream_t s) {
    k_import<T><<<(n + 255) / 256, 256, 0, s>>>(n, perm, wfile, W);
}

template <typename T>
void enqueue_export(int n, const int *perm, const V4<T> *W, double *wfile, cudaStream_t s) {
    k_export<T><<<(n + 255) / 256, 256, 0, s>>>(n, perm, W, wfile);
}

// ---------------------------------------------------------------------------
// One iteration: gpu_solver.cu:2200-2434 without the W -> W0 copies.  W[0]
// holds the start state; stage 0 reads it and writes W[1], middle stages
// update W[1] in place, and the last stage writes the result back into W[0]
// (each cell reads its own W0 before overwriting it), so W[0] is also the
// next iteration's W0.
template <typename T> void enqueue_iteration(const Plan<T> &p, cudaStream_t s) {
    const int n = p.m.n, B = p.block, G = (n + B - 1) / B;
    const bool opt = faces_options(p.f, p.phi);
    for (int st = 0; st < p.stages; st++) {
        const bool last = st == p.stages - 1;
        V4<T> *Wcur = st == 0 ? p.W[0] : p.W[1];
        V4<T> *Wout = last ? p.W[0] : p.W[1];
        if (opt) launch_chained(k_faces<T, true>, G, B, s, p.m, p.f, Wcur, p.FS, p.dt, p.ctl, p.phi, st);
        else if (faces_tiled<T>(B))
            launch_chained(k_faces_tile<T>, G, B, s, p.m, p.f, Wcur, p.FS, p.dt, p.ctl, p.phi, st);
        else launch_chained(k_faces<T, false>, G, B, s, p.m, p.f, Wcur, p.FS, p.dt, p.ctl, p.phi, st);
        if (FluxTiled<T>::value) launch_chained(k_flux_tile<T>, G, B, s, p.m, p.f, p.FS, p.res, p.ctl);
        else launch_chained(k_flux<T>, G, B, s, p.m, p.f, p.FS, p.res, p.ctl);
        const V4<T> *src = p.res;
        for (int sw = 0; sw + 1 < p.sweeps; sw++) {
            V4<T> *dst = p.sm[sw & 1];
            launch_chained(k_smooth<T>, G, B, s, p.m, p.f.irs_eps, src, p.res, dst, p.ctl);
            src = dst;
        }
        if (p.f.global_dt)
            launch_chained(k_update<T, true>, G, B, s, p.m, p.f, p.rk[st], p.sweeps > 0 ? 1 : 0, src, p.res, p.dt,
                           p.W[0], Wout, last ? p.part : nullptr, p.ctl, st);
        else
            launch_chained(k_update<T, false>, G, B, s, p.m, p.f, p.rk[st], p.sweeps > 0 ? 1 : 0, src, p.res, p.dt,
                           p.W[0], Wout, last ? p.part : nullptr, p.ctl, st);
    }
    enqueue_resid(p.part, G, p.ctl, p.hist, p.hist_cap, sizeof(T) == 4, s);
}

// Same launches as enqueue_iteration, with events recorded around each one.
// ev[2*j], ev[2*j+1] bracket launch j; kind[j] is 0 faces, 1 flux, 2 smooth,
// 3 update, 4 resid.  Returns the number of launches.
template <typename T>
int enqueue_iteration_timed(const Plan<T> &p, cudaStream_t s, cudaEvent_t *ev, int *kind) {
    const int n = p.m.n, B = p.block, G = (n + B - 1) / B;
    const bool opt = faces_options(p.f, p.phi);
    int j = 0;
    auto mark = [&](int k) { kind[j] = k; cudaEventRecord(ev[2 * j], s); };
    auto done = [&]() { cudaEventRecord(ev[2 * j + 1], s); j++; };
    for (int st = 0; st < p.stages; st++) {
        const bool last = st == p.stages - 1;
        V4<T> *Wcur = st == 0 ? p.W[0] : p.W[1];
        V4<T> *Wout = last ? p.W[0] : p.W[1];
        mark(0);
        if (opt) k_faces<T, true><<<G, B, 0, s>>>(p.m, p.f, Wcur, p.FS, p.dt, p.ctl, p.phi, st);
        else if (faces_tiled<T>(B)) k_faces_tile<T><<<G, B, 0, s>>>(p.m, p.f, Wcur, p.FS, p.dt, p.ctl, p.phi, st);
        else k_faces<T, false><<<G, B, 0, s>>>(p.m, p.f, Wcur, p.FS, p.dt, p.ctl, p.phi, st);
        done();
        mark(1);
        if (FluxTiled<T>::value) k_flux_tile<T><<<G, B, 0, s>>>(p.m, p.f, p.FS, p.res, p.ctl);
        else k_flux<T><<<G, B, 0, s>>>(p.m, p.f, p.FS, p.res, p.ctl);
        done();
        const V4<T> *src = p.res;
        for (int sw = 0; sw + 1 < p.sweeps; sw++) {
            V4<T> *dst = p.sm[sw & 1];
            mark(2); k_smooth<T><<<G, B, 0, s>>>(p.m, p.f.irs_eps, src, p.res, dst, p.ctl); done();
            src = dst;
        }
        mark(3);
        if (p.f.global_dt)
            k_update<T, true><<<G, B, 0, s>>>(p.m, p.f, p.rk[st], p.sweeps > 0 ? 1 : 0, src, p.res, p.dt,
                                              p.W[0], Wout, last ? p.part : nullptr, p.ctl, st);
        else
            k_update<T, false><<<G, B, 0, s>>>(p.m, p.f, p.rk[st], p.sweeps > 0 ? 1 : 0, src, p.res, p.dt,
                                               p.W[0], Wout, last ? p.part : nullptr, p.ctl, st);
        done();
    }
    mark(4); enqueue_resid(p.part, G, p.ctl, p.hist, p.hist_cap, sizeof(T) == 4, s); done();
    return j;
}

}  // namespace e2d
