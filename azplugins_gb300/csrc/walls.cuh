// walls.cuh -- wall potentials (src/WallEvaluatorLJ93.h, src/WallEvaluatorColloid.h)
// over HOOMD's wall geometries (spheres, cylinders, planes), as HOOMD's
// EvaluatorWalls applies a wall evaluator (restated from its documented
// behaviour; it is not part of the azplugins tree).
//
// For each wall: dr = the particle minus the nearest point of the wall surface,
// and whether the particle is on the wall's active side ("inside"). Standard mode
// (r_extrap = 0): the energy-shifted evaluator at |dr| on the active side only.
// Extrapolated mode (r_extrap > 0): the evaluator where the particle is on the
// active side at least r_extrap from the surface, elsewhere the linear
// continuation U(r_extrap) + F(r_extrap) (r_extrap - d) with d the signed
// distance (negative on the inactive side) and the constant force F(r_extrap)
// directed towards the active side. Energies are whole (no pair halving); the
// virial is F_a x_b.
#pragma once

#include <cmath>
#include <cstdint>

#include "common.cuh"

namespace azp
{
// limits of HOOMD's wall field (MAX_N_SWALLS, MAX_N_CWALLS, MAX_N_PWALLS)
constexpr int WALL_MAX_SPHERES = AZP_WALL_MAX_SPHERES;
constexpr int WALL_MAX_CYLINDERS = AZP_WALL_MAX_CYLINDERS;
constexpr int WALL_MAX_PLANES = AZP_WALL_MAX_PLANES;

struct WallSphereD {
    double r, o[3];
    int inside, open;
};
struct WallCylinderD {
    double r, o[3], ax[3];  // ax: unit axis
    int inside, open;
};
struct WallPlaneD {
    double o[3], n[3];  // n: unit normal (the active side)
    int open, pad_;
};
// passed by value as a kernel argument (read from the constant bank)
struct WallField {
    int ns, nc, np, pad_;
    WallSphereD s[WALL_MAX_SPHERES];
    WallCylinderD c[WALL_MAX_CYLINDERS];
    WallPlaneD p[WALL_MAX_PLANES];
};

// ---------------------------------------------------------------- evaluators
// src/WallEvaluatorLJ93.h:100-133: p = {sigma^3, A}; energy shifted at r_cut
struct WallLJ93 {
    AZP_HD static bool eval(const double* p, double rsq, double rcutsq, double& fdr, double& e)
    {
        const double lj1 = (2.0 / 15.0) * p[1] * p[0] * p[0] * p[0];
        const double lj2 = p[1] * p[0];
        if (!(rsq < rcutsq) || lj1 == 0.0) return false;
        const double r2inv = 1.0 / rsq;
        const double r3inv = r2inv * sqrt(r2inv);
        const double r6inv = r3inv * r3inv;
        fdr = r2inv * r3inv * (9.0 * lj1 * r6inv - 3.0 * lj2);
        e = r3inv * (lj1 * r6inv - lj2);
        const double rc2inv = 1.0 / rcutsq;
        const double rc3inv = rc2inv * sqrt(rc2inv);
        const double rc6inv = rc3inv * rc3inv;
        e -= rc3inv * (lj1 * rc6inv - lj2);
        return true;
    }
};

// src/WallEvaluatorColloid.h:118-183: p = {c_1, c_2, a}; energy shifted at r_cut
struct WallColloid {
    AZP_HD static double potential(const double* p, double rsq, bool force, double& fdr)
    {
        const double c1 = p[0], c2 = p[1], a = p[2];
        const double r = sqrt(rsq);
        const double arinv = a / r;
        const double rma = 1.0 / (r - a), rpa = 1.0 / (r + a);
        const double r2ma2 = rma * rpa;
        const double rma2 = rma * rma, rma6 = rma2 * rma2 * rma2;
        const double rpa2 = rpa * rpa, rpa6 = rpa2 * rpa2 * rpa2;
        if (force) {
            const double arinv8 = 8.0 * arinv;
            fdr = 6.0 * c1 * ((arinv8 - 1.0) * rma2 * rma6 + (arinv8 + 1.0) * rpa2 * rpa6);
            fdr -= c2 * (4.0 * a * a * arinv * r2ma2 * r2ma2);
        }
        const double a7 = 7.0 * a;
        double en = c1 * ((a7 - r) * rma * rma6 + (a7 + r) * rpa * rpa6);
        en -= c2 * (2.0 * a * r * r2ma2 + log(rpa / rma));
        return en;
    }
    AZP_HD static bool eval(const double* p, double rsq, double rcutsq, double& fdr, double& e)
    {
        if (!(rsq < rcutsq) || p[0] == 0.0 || !(p[2] > 0.0)) return false;
        double unused = 0.0;
        e = potential(p, rsq, true, fdr) - potential(p, rcutsq, false, unused);
        return true;
    }
};

// ---------------------------------------------------------------- geometry
// dr = x - nearest surface point; nrm = unit normal towards the active side at
// that point (used when the particle lies exactly on the surface)
AZP_HD void wall_sphere(const WallSphereD& w, const double* x, double* dr, double* nrm, bool& inside)
{
    const double t[3] = {x[0] - w.o[0], x[1] - w.o[1], x[2] - w.o[2]};
    const double rxyz = sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
    if (rxyz > 0.0) {
        inside = (w.inside ? rxyz < w.r : rxyz > w.r) || (rxyz == w.r && !w.open);
        // one reciprocal instead of four divisions (FP64 division is slow here)
        const double rinv = 1.0 / rxyz;
        const double s = w.r * rinv;
        for (int d = 0; d < 3; ++d) {
            dr[d] = t[d] - t[d] * s;
            nrm[d] = w.inside ? -t[d] * rinv : t[d] * rinv;
        }
    } else {
        // at the centre every surface point is nearest: the one along +x
        inside = w.inside != 0;
        dr[0] = -w.r;
        dr[1] = dr[2] = 0.0;
        nrm[0] = nrm[1] = nrm[2] = 0.0;
    }
}

AZP_HD void wall_cylinder(const WallCylinderD& w, const double* x, double* dr, double* nrm, bool& inside)
{
    const double t[3] = {x[0] - w.o[0], x[1] - w.o[1], x[2] - w.o[2]};
    const double along = t[0] * w.ax[0] + t[1] * w.ax[1] + t[2] * w.ax[2];
    const double pp[3] = {t[0] - along * w.ax[0], t[1] - along * w.ax[1], t[2] - along * w.ax[2]};
    const double rxy = sqrt(pp[0] * pp[0] + pp[1] * pp[1] + pp[2] * pp[2]);
    if (rxy > 0.0) {
        inside = (w.inside ? rxy < w.r : rxy > w.r) || (rxy == w.r && !w.open);
        const double rinv = 1.0 / rxy;
        const double s = w.r * rinv;
        for (int d = 0; d < 3; ++d) {
            dr[d] = pp[d] - pp[d] * s;
            nrm[d] = w.inside ? -pp[d] * rinv : pp[d] * rinv;
        }
    } else {
        // on the axis: the surface point along the first direction normal to the axis
        inside = w.inside != 0;
        double u[3];
        if (fabs(w.ax[0]) < 0.9) {
            u[0] = 0.0;
            u[1] = w.ax[2];
            u[2] = -w.ax[1];
        } else {
            u[0] = -w.ax[2];
            u[1] = 0.0;
            u[2] = w.ax[0];
        }
        const double un = sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (int d = 0; d < 3; ++d) {
            dr[d] = -w.r * u[d] / un;
            nrm[d] = 0.0;
        }
    }
}

AZP_HD void wall_plane(const WallPlaneD& w, const double* x, double* dr, double* nrm, bool& inside)
{
    const double d = (x[0] - w.o[0]) * w.n[0] + (x[1] - w.o[1]) * w.n[1] + (x[2] - w.o[2]) * w.n[2];
    inside = d > 0.0 || (d == 0.0 && !w.open);
    for (int k = 0; k < 3; ++k) {
        dr[k] = d * w.n[k];
        nrm[k] = w.n[k];
    }
}

// one wall's force and energy added to (F, U)
template<class EV>
AZP_HD void wall_apply(const double* p, double rcutsq, double rextrap, const double* dr, const double* nrm,
                       bool inside, double* F, double& U)
{
    const double rsq = dr[0] * dr[0] + dr[1] * dr[1] + dr[2] * dr[2];
    double fdr = 0.0, e = 0.0;
    if (rextrap > 0.0) {
        const double rextrapsq = rextrap * rextrap;
        if (inside && rsq >= rextrapsq) {
            if (EV::eval(p, rsq, rcutsq, fdr, e)) {
                for (int d = 0; d < 3; ++d) F[d] += dr[d] * fdr;
                U += e;
            }
            return;
        }
        const double r = sqrt(rsq);
        double u[3];
        if (rsq > 0.0) {
            const double sr = (inside ? 1.0 : -1.0) / r;
            for (int d = 0; d < 3; ++d) u[d] = sr * dr[d];
        } else {
            for (int d = 0; d < 3; ++d) u[d] = nrm[d];
        }
        const double rp = inside ? rextrap - r : rextrap + r;
        if (EV::eval(p, rextrapsq, rcutsq, fdr, e)) {
            const double fmag = fdr * rextrap;
            for (int d = 0; d < 3; ++d) F[d] += u[d] * fmag;
            U += e + fmag * rp;
        }
        return;
    }
    if (!inside) return;
    if (EV::eval(p, rsq, rcutsq, fdr, e)) {
        for (int d = 0; d < 3; ++d) F[d] += dr[d] * fdr;
        U += e;
    }
}

// all walls: spheres, then cylinders, then planes
template<class EV>
AZP_HD void walls_force(const WallField& wf, const double* p, double rcutsq, double rextrap, const double* x,
                        double* F, double& U)
{
    double dr[3], nrm[3];
    bool inside = false;
    for (int k = 0; k < wf.ns; ++k) {
        wall_sphere(wf.s[k], x, dr, nrm, inside);
        wall_apply<EV>(p, rcutsq, rextrap, dr, nrm, inside, F, U);
    }
    for (int k = 0; k < wf.nc; ++k) {
        wall_cylinder(wf.c[k], x, dr, nrm, inside);
        wall_apply<EV>(p, rcutsq, rextrap, dr, nrm, inside, F, U);
    }
    for (int k = 0; k < wf.np; ++k) {
        wall_plane(wf.p[k], x, dr, nrm, inside);
        wall_apply<EV>(p, rcutsq, rextrap, dr, nrm, inside, F, U);
    }
}

// ---------------------------------------------------------------- FP32 screen
// True when some wall may act on a particle at (x, y, z): its float distance d
// to a wall, positive on the active side, lies below reach (= max(r_cut,
// r_extrap) + tol) and, without extrapolation, above -tol. tol bounds the float
// error of d, so a false answer is exact: walls_force would add nothing (the
// reach test covers both branches of wall_apply, the sign test its inside flag).
#ifdef __CUDACC__
__device__ __forceinline__ bool walls_near(const WallField& wf, float reach, bool extrap, float x, float y, float z,
                                           float tol)
{
    for (int k = 0; k < wf.ns; ++k) {
        const WallSphereD& w = wf.s[k];
        const float dx = x - (float)w.o[0], dy = y - (float)w.o[1], dz = z - (float)w.o[2];
        const float r = sqrtf(dx * dx + dy * dy + dz * dz);
        const float d = w.inside ? (float)w.r - r : r - (float)w.r;
        if (d < reach && (extrap || d > -tol)) return true;
    }
    for (int k = 0; k < wf.nc; ++k) {
        const WallCylinderD& w = wf.c[k];
        const float dx = x - (float)w.o[0], dy = y - (float)w.o[1], dz = z - (float)w.o[2];
        const float al = dx * (float)w.ax[0] + dy * (float)w.ax[1] + dz * (float)w.ax[2];
        const float px = dx - al * (float)w.ax[0], py = dy - al * (float)w.ax[1], pz = dz - al * (float)w.ax[2];
        const float r = sqrtf(px * px + py * py + pz * pz);
        const float d = w.inside ? (float)w.r - r : r - (float)w.r;
        if (d < reach && (extrap || d > -tol)) return true;
    }
    for (int k = 0; k < wf.np; ++k) {
        const WallPlaneD& w = wf.p[k];
        const float d = (x - (float)w.o[0]) * (float)w.n[0] + (y - (float)w.o[1]) * (float)w.n[1] +
                        (z - (float)w.o[2]) * (float)w.n[2];
        if (d < reach && (extrap || d > -tol)) return true;
    }
    return false;
}

// The screen's tolerance for a caller's FP64 position x: the float rounding of
// x, of the wall origins, radii, axes and normals, and of the few operations
// between them stays below 64 units of 2^-24 of |x|_1 + mag, where mag is the
// largest |origin|_1 + radius over the walls plus the type's reach (a bound
// with room to spare: the cylinder's projection, the longest chain, needs about
// 40 such units). A position whose float magnitude is not finite gets an
// infinite tolerance, so that the screen passes it on to the FP64 evaluation.
__device__ __forceinline__ float walls_screen_tol(const double* x, float mag)
{
    const float m = fabsf((float)x[0]) + fabsf((float)x[1]) + fabsf((float)x[2]);
    return m < 1.0e37f ? 0x1p-18f * (m + mag) + 1.0e-30f : INFINITY;
}
#endif

// ---------------------------------------------------------------- FP32 path
// Per-type float record of the FP32 driver, made once per block from the FP64
// evaluator: q[0..2] the evaluator's constants (LJ93: lj1 = 2/15 A sigma^9,
// lj2 = A sigma^3; Colloid: c_1, c_2, a), q[3] the energy at r_cut (the shift),
// q[4] r_cut^2, q[5] the force magnitude F(r_extrap) = (F/r)(r_extrap) r_extrap,
// q[6] U(r_extrap) (shifted), q[7] r_extrap.
constexpr int WALL_F = 8;

template<class EV> AZP_D void wall_record_f(const double* p, double rc, double rx, float* q);

template<> AZP_D void wall_record_f<WallLJ93>(const double* p, double rc, double rx, float* q)
{
    const double lj1 = (2.0 / 15.0) * p[1] * p[0] * p[0] * p[0], lj2 = p[1] * p[0];
    const double rc2 = rc * rc;
    const double rc2inv = 1.0 / rc2, rc3inv = rc2inv * sqrt(rc2inv), rc6inv = rc3inv * rc3inv;
    q[0] = (float)lj1;
    q[1] = (float)lj2;
    q[2] = 0.0f;
    q[3] = (float)(rc3inv * (lj1 * rc6inv - lj2));
    q[4] = (float)rc2;
    double fdr = 0.0, e = 0.0;
    const bool ok = rx > 0.0 && WallLJ93::eval(p, rx * rx, rc2, fdr, e);
    q[5] = ok ? (float)(fdr * rx) : 0.0f;
    q[6] = ok ? (float)e : 0.0f;
    q[7] = (float)rx;
}

template<> AZP_D void wall_record_f<WallColloid>(const double* p, double rc, double rx, float* q)
{
    const double rc2 = rc * rc;
    double unused = 0.0;
    q[0] = (float)p[0];
    q[1] = (float)p[1];
    q[2] = (float)p[2];
    q[3] = (p[0] != 0.0 && p[2] > 0.0) ? (float)WallColloid::potential(p, rc2, false, unused) : 0.0f;
    q[4] = (float)rc2;
    double fdr = 0.0, e = 0.0;
    const bool ok = rx > 0.0 && WallColloid::eval(p, rx * rx, rc2, fdr, e);
    q[5] = ok ? (float)(fdr * rx) : 0.0f;
    q[6] = ok ? (float)e : 0.0f;
    q[7] = (float)rx;
}

// FP32 evaluators on the float record (the same forms as the FP64 ones)
struct WallLJ93F {
    AZP_D static bool eval(const float* q, float rsq, float& fdr, float& e)
    {
        if (!(rsq < q[4]) || q[0] == 0.0f) return false;
        const float r2inv = 1.0f / rsq;
        const float r3inv = r2inv * sqrtf(r2inv);
        const float r6inv = r3inv * r3inv;
        fdr = r2inv * r3inv * (9.0f * q[0] * r6inv - 3.0f * q[1]);
        e = r3inv * (q[0] * r6inv - q[1]) - q[3];
        return true;
    }
};

struct WallColloidF {
    AZP_D static bool eval(const float* q, float rsq, float& fdr, float& e)
    {
        const float c1 = q[0], c2 = q[1], a = q[2];
        if (!(rsq < q[4]) || c1 == 0.0f || !(a > 0.0f)) return false;
        const float r = sqrtf(rsq);
        const float arinv = a / r;
        const float rma = 1.0f / (r - a), rpa = 1.0f / (r + a);
        const float r2ma2 = rma * rpa;
        const float rma2 = rma * rma, rma6 = rma2 * rma2 * rma2;
        const float rpa2 = rpa * rpa, rpa6 = rpa2 * rpa2 * rpa2;
        const float arinv8 = 8.0f * arinv;
        fdr = 6.0f * c1 * ((arinv8 - 1.0f) * rma2 * rma6 + (arinv8 + 1.0f) * rpa2 * rpa6) -
              c2 * (4.0f * a * a * arinv * r2ma2 * r2ma2);
        const float a7 = 7.0f * a;
        e = c1 * ((a7 - r) * rma * rma6 + (a7 + r) * rpa * rpa6) - c2 * (2.0f * a * r * r2ma2 + logf(rpa / rma)) - q[3];
        return true;
    }
};

// one wall in FP32 from its distance d >= 0, the unit vector u from the nearest
// surface point to the particle (dr = d u), the active-side flag and the surface
// normal towards the active side (used at d = 0)
template<class EVF>
AZP_D void wall_apply_f(const float* q, float d, const float* u, bool inside, const float* nrm, float* F, float& U)
{
    const float rx = q[7];
    float fdr = 0.0f, e = 0.0f;
    if (rx > 0.0f) {
        if (inside && d >= rx) {
            if (EVF::eval(q, d * d, fdr, e)) {
                for (int k = 0; k < 3; ++k) F[k] += u[k] * (d * fdr);
                U += e;
            }
            return;
        }
        // linear continuation: constant force towards the active side
        const float sgn = inside ? 1.0f : -1.0f;
        const float* dir = d > 0.0f ? u : nrm;
        const float s = d > 0.0f ? sgn : 1.0f;
        for (int k = 0; k < 3; ++k) F[k] += s * dir[k] * q[5];
        U += q[6] + q[5] * (rx - sgn * d);
        return;
    }
    if (!inside) return;
    if (EVF::eval(q, d * d, fdr, e)) {
        for (int k = 0; k < 3; ++k) F[k] += u[k] * (d * fdr);
        U += e;
    }
}

// a curved wall (sphere: axis = nullptr; cylinder: unit axis) in FP32 with the
// FP64 parts that cancellation needs: x - origin, r^2 and R^2 - r^2, so that the
// distance R - r = (R^2 - r^2) / (R + r) keeps FP32 relative accuracy near the
// surface without an FP64 square root
template<class EVF>
AZP_D void curved_wall_f(double R, const double* o, const double* ax, int w_inside, int w_open, const double* x,
                         const float* q, float* F, float& U)
{
    double t[3] = {x[0] - o[0], x[1] - o[1], x[2] - o[2]};
    if (ax) {
        const double al = t[0] * ax[0] + t[1] * ax[1] + t[2] * ax[2];
        for (int k = 0; k < 3; ++k) t[k] -= al * ax[k];
    }
    const double r2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    float u[3], nrm[3], d;
    bool inside;
    if (r2 > 0.0) {
        const float rf = sqrtf((float)r2);
        const float din = (float)(R * R - r2) / ((float)R + rf);  // R - r, > 0 inside the surface
        const float rinv = 1.0f / rf;
        const float th[3] = {(float)t[0] * rinv, (float)t[1] * rinv, (float)t[2] * rinv};
        inside = (w_inside ? din > 0.0f : din < 0.0f) || (din == 0.0f && !w_open);
        d = fabsf(din);
        const float sd = din > 0.0f ? -1.0f : 1.0f;  // from the surface point to the particle
        for (int k = 0; k < 3; ++k) {
            u[k] = sd * th[k];
            nrm[k] = w_inside ? -th[k] : th[k];
        }
    } else {
        // at the centre (on the axis): the surface point along a fixed direction, as in the FP64 path
        double dir[3] = {1.0, 0.0, 0.0};
        if (ax) {
            if (fabs(ax[0]) < 0.9) {
                dir[0] = 0.0;
                dir[1] = ax[2];
                dir[2] = -ax[1];
            } else {
                dir[0] = -ax[2];
                dir[1] = 0.0;
                dir[2] = ax[0];
            }
            const double un = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
            for (int k = 0; k < 3; ++k) dir[k] /= un;
        }
        inside = w_inside != 0;
        d = (float)R;
        for (int k = 0; k < 3; ++k) {
            u[k] = -(float)dir[k];
            nrm[k] = 0.0f;
        }
    }
    wall_apply_f<EVF>(q, d, u, inside, nrm, F, U);
}

template<class EVF>
AZP_D void walls_force_f(const WallField& wf, const float* q, const double* x, float* F, float& U)
{
    for (int k = 0; k < wf.ns; ++k)
        curved_wall_f<EVF>(wf.s[k].r, wf.s[k].o, nullptr, wf.s[k].inside, wf.s[k].open, x, q, F, U);
    for (int k = 0; k < wf.nc; ++k)
        curved_wall_f<EVF>(wf.c[k].r, wf.c[k].o, wf.c[k].ax, wf.c[k].inside, wf.c[k].open, x, q, F, U);
    for (int k = 0; k < wf.np; ++k) {
        const WallPlaneD& w = wf.p[k];
        const float ds = (float)((x[0] - w.o[0]) * w.n[0] + (x[1] - w.o[1]) * w.n[1] + (x[2] - w.o[2]) * w.n[2]);
        const bool inside = ds > 0.0f || (ds == 0.0f && !w.open);
        const float nrm[3] = {(float)w.n[0], (float)w.n[1], (float)w.n[2]};
        const float sg = ds < 0.0f ? -1.0f : 1.0f;
        const float u[3] = {sg * nrm[0], sg * nrm[1], sg * nrm[2]};
        wall_apply_f<EVF>(q, fabsf(ds), u, inside, nrm, F, U);
    }
}

// host: the C-ABI wall list as a WallField (axes and normals normalised, as
// HOOMD's wall constructors do); AZP_ERR_INVALID on a bad wall or count
int make_wall_field(const azp_walls* walls, WallField* out);

// host: the largest |origin|_1 + |radius| over the field's walls (the wall part
// of the FP32 screen's tolerance)
float wall_field_extent(const WallField& wf);

}  // namespace azp
