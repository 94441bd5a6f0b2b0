// integrals.cu -- FP64 integrals of a conserved state, on the host: lift and
// drag (forces_from_state), total mass, and the mass fluxes through the
// far-field and wall faces.  No reference counterpart.
//
// The boundary fluxes are the scheme's own first-order boundary flux, the one
// the kernels evaluate for a boundary face (the interior cell's state against
// its ghost, no reconstruction), restated here in FP64 in the reference's
// operation order; built without contraction, each face gives the bits of the
// FP64 kernels.  Only the mass component of the Roe flux is formed.
#include <cmath>
#include <string>
#include <vector>

#include "solver_internal.h"

namespace e2d {
namespace {

constexpr double kGasR = 287.06;  // gpu_init.cu:69 (R of the far-field ghost)

struct Cons {
    double r, ru, rv, re;
};

// gpu_solver.cu:49-60 (kernel_CalculationPTA): pressure and sound speed.
void pressure_sound(const Cons &w, double g, double &P, double &A) {
    double U = w.ru / w.r;
    double V = w.rv / w.r;
    double E = w.re / w.r - 0.5 * (U * U + V * V);
    P = (g - 1.0) * w.r * E;
    A = std::sqrt(g * P / w.r);
}

// gpu_solver.cu:62-135 (kernel_Far_Boundary) for the face vector
// (vectorx, vectory) of an interior state dw.
Cons far_ghost(const Cons &dw, double vectorx, double vectory, const FreeStream &fs, const e2d_params &p) {
    const double g = p.gamma;
    double P, A;
    pressure_sound(dw, g, P, A);
    double nn = std::sqrt(vectorx * vectorx + vectory * vectory);
    double nx = vectory / nn;
    double ny = vectorx / nn;
    double UD = dw.ru / dw.r;
    double VD = dw.rv / dw.r;
    double Un = std::fabs(fs.ui * nx + fs.vi * ny);
    double Uncell = UD * nx + VD * ny;
    Cons w0 = dw;
    if (Un / fs.ain_test > 1.0) {
        if (!(Uncell > 0.0)) {
            w0.r = 1.0;
            w0.ru = fs.ui;
            w0.rv = fs.vi;
            w0.re = kGasR * p.tin / (fs.vin * fs.vin) / (g - 1.0) + 0.50;
        }
    } else {
        double PA = fs.pis, PD = P, AD = A, ROUD = dw.r, PB, UB, VB;
        if (Uncell > 0.0) {
            PB = PA;
            w0.r = ROUD + (PB - PD) / AD / AD;
            UB = UD + nx * (PD - PB) / ROUD / AD;
            VB = VD + ny * (PD - PB) / ROUD / AD;
        } else {
            PB = 0.5 * (PA + PD - ROUD * AD * (nx * (fs.ui - UD) + ny * (fs.vi - VD)));
            w0.r = 1.0 + (PB - PA) / AD / AD;
            UB = fs.ui - nx * (PA - PB) / ROUD / AD;
            VB = fs.vi - ny * (PA - PB) / ROUD / AD;
        }
        w0.ru = UB * w0.r;
        w0.rv = VB * w0.r;
        w0.re = PB / (g - 1.0) + 0.5 * (UB * UB + VB * VB) * w0.r;
    }
    return w0;
}

// gpu_solver.cu:188-221: slip-wall ghost, the velocity mirrored in the face.
Cons wall_ghost(const Cons &dw, double vectorx, double vectory, double vectorn) {
    double nij0 = vectory / vectorn;
    double nij1 = vectorx / vectorn;
    double UU = dw.ru / dw.r;
    double VV = dw.rv / dw.r;
    double UV = UU * nij0 + VV * nij1;
    UU = UU - 2.0 * UV * nij0;
    VV = VV - 2.0 * UV * nij1;
    Cons o = dw;
    o.ru = dw.r * UU;
    o.rv = dw.r * VV;
    return o;
}

// gpu_solver.cu:552-566 (kernel_Calc_Function)
void calc_function(const Cons &w, double g, double &A, double &U, double &V, double &H, double &P) {
    double temp = 1.0 / w.r;
    U = w.ru * temp;
    V = w.rv * temp;
    P = (g - 1.0) * w.r * (w.re * temp - 0.5 * (U * U + V * V));
    A = std::sqrt(g * P * temp);
    H = w.re * temp + P * temp;
}

// Mass component of the Roe flux with Harten's entropy fix of width eps
// through the unit normal (nx, ny), gpu_solver.cu:569-647.
double roe_mass(const Cons &LW, const Cons &RW, double nx, double ny, double g, double epsilon) {
    double A0, U0, V0, H0, P0, A1, U1, V1, H1, P1;
    calc_function(LW, g, A0, U0, V0, H0, P0);
    calc_function(RW, g, A1, U1, V1, H1, P1);
    double M0 = (U0 * nx + V0 * ny);
    double M1 = (U1 * nx + V1 * ny);
    double DVC = M1 - M0;
    double lrou = LW.r, rrou = RW.r;
    double sl = std::sqrt(lrou), sr = std::sqrt(rrou);
    double ROUB = sl * sr;
    double UB = (U0 * sl + U1 * sr) / (sl + sr);
    double VB = (V0 * sl + V1 * sr) / (sl + sr);
    double HB = (H0 * sl + H1 * sr) / (sl + sr);
    double QB = UB * UB + VB * VB;
    double AB = std::sqrt((g - 1.0) * (HB - QB / 2.0));
    double VC = UB * nx + VB * ny;
    double AD0, AD1, AD2;
    if (std::fabs(VC - AB) < epsilon) AD0 = ((VC - AB) * (VC - AB) + epsilon * epsilon) / (2.0 * epsilon);
    else AD0 = std::fabs(VC - AB);
    if (std::fabs(VC) < epsilon) AD1 = (VC * VC + epsilon * epsilon) / (2.0 * epsilon);
    else AD1 = std::fabs(VC);
    if (std::fabs(VC + AB) < epsilon) AD2 = ((VC + AB) * (VC + AB) + epsilon * epsilon) / (2.0 * epsilon);
    else AD2 = std::fabs(VC + AB);
    double dP = P1 - P0;
    double F00 = AD0 * (dP - ROUB * AB * DVC) / (2.0 * AB * AB);
    double F10 = AD1 * ((rrou - lrou) - dP / (AB * AB));
    double F20 = AD2 * (dP + ROUB * AB * DVC) / (2.0 * AB * AB);
    double WL0 = lrou * M0;
    double WR0 = rrou * M1;
    return 0.5 * ((WL0 + WR0) - (F00 + F10 + F20));
}

}  // namespace

void integrals_from_state(const HostLayout &L, const FreeStream &fs, const e2d_params &p, const double *w,
                          e2d_integrals *out) {
    forces_from_state(L, fs, p.gamma, w, &out->cl, &out->cd);
    const int n = L.n;
    double mass = 0.0, far = 0.0, wall = 0.0;
    for (int i = 0; i < n; i++) {
        const double *u = &w[4 * (size_t)L.perm[i]];
        const Cons c{u[0], u[1], u[2], u[3]};
        mass += c.r * L.area[i];
        for (int k = 0; k < 3; k++) {
            const int code = L.topo[4 * (size_t)i + k];
            if (code >= 0) continue;
            // S = (vectory, vectorx), outward from the interior cell; as the
            // kernels' face flux: n = S / |S|, flux times |S|
            const double Sx = L.S[2 * ((size_t)k * n + i)], Sy = L.S[2 * ((size_t)k * n + i) + 1];
            const double vn = std::sqrt(Sy * Sy + Sx * Sx);
            const double nx = Sx / vn, ny = Sy / vn;
            Cons b;
            if (code == -1) b = far_ghost(c, Sy, Sx, fs, p);
            else b = wall_ghost(c, Sy, Sx, std::sqrt(Sy * Sy + Sx * Sx));
            const double f = roe_mass(c, b, nx, ny, p.gamma, p.entropy_eps) * vn;
            (code == -1 ? far : wall) += f;
        }
    }
    out->mass = mass;
    out->mass_flux_far = far;
    out->mass_flux_wall = wall;
}

}  // namespace e2d

using namespace e2d;

extern "C" int e2d_state_integrals(e2d_mesh *m, const e2d_params *p, const double *w, e2d_integrals *out) {
    if (!m || !p || !w || !out) { set_error("null argument"); return E2D_ERR_ARG; }
    if (const char *why = param_error(p)) { set_error(std::string("invalid parameters: ") + why); return E2D_ERR_ARG; }
    HostLayout L;
    int rc = build_layout(m, *p, L);
    if (rc) return rc;
    integrals_from_state(L, free_stream(*p), *p, w, out);
    return E2D_OK;
}
