// Host-side construction of the reference's tabulated potentials.
//
// Tissue Forge stores every nonbonded and bonded potential as a piecewise quintic
// interpolation table built once on the host (potential_init, source/mdcore/src/
// tfPotential.cpp:1396-1634).  The GPU engine consumes those tables verbatim, so this
// file restates the construction with the reference's single-precision build types
// (FPTYPE = float, CMakeLists.txt:244-253): float state, double intermediates exactly
// where the reference's C++ expressions promote to double, and no FMA contraction
// (this file is compiled with -ffp-contract=off).
//
// Promotion rule: tfPotential.cpp includes <cmath> but never <math.h>, so its
// unqualified fabs/sqrt/cos/acos calls on float arguments resolve to the C library's
// double functions; only explicitly qualified std:: calls (Power(), std::sqrt in
// DPDPotential) take the float overloads.  The domain stretch, the transform correction
// and the harmonic-angle interpoland below therefore compute in double.
//
// Steps restated (same order, same arithmetic types):
//   node density transform        potential_getalpha      tfPotential.cpp:1977-2040
//   node placement (Newton)                               tfPotential.cpp:1457-1465
//   first derivatives at nodes    potential_getfp         tfPotential.cpp:1650-1731
//                                 potential_getfp_fixend  tfPotential.cpp:1734-1815
//   per-interval coefficients     potential_getcoeffs     tfPotential.cpp:1839-1961
//   interval-count bisection                              tfPotential.cpp:1509-1598
//   linear continuation of [0]                            tfPotential.cpp:1609-1624
// Factories: Morse :2193-2283, LJ 12-6 :192-245/1087-1109, harmonic :344-401,
// harmonic angle :554-626, DPD tfDPDPotential.cpp:32-43.
#include "tfg.h"

#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <vector>

namespace {

typedef float real;                       // FPTYPE of the reference's CUDA-enabled build
constexpr int kDegree = 5;                // potential_degree
constexpr int kChunk = kDegree + 3;       // potential_chunk
constexpr int kIvalsA = 1;                // potential_ivalsa
constexpr int kIvalsB = 10;               // potential_ivalsb
constexpr int kSamples = 100;             // potential_N
constexpr int kIvalsMax = 3048;           // potential_ivalsmax
const double kPi = 3.14159265358979323846;

// The function being tabulated, its first derivative (may be empty) and its sixth
// derivative (drives the node distribution).
struct Interpoland {
    std::function<real(real)> f, fp, f6p;
};

// Chebyshev-Lobatto sample weights shared by both derivative solvers.
struct LobattoWeights {
    real xi[kSamples], w[kSamples];
    LobattoWeights() {
        for (int k = 1; k < kSamples - 1; k++) {
            xi[k] = std::cos(k * kPi / (kSamples - 1));
            w[k] = 1.0 / std::sqrt(1.0 - xi[k] * xi[k]);
        }
        xi[0] = 1.0; xi[kSamples - 1] = -1.0;
        w[0] = 0.0; w[kSamples - 1] = 0.0;
    }
};
const LobattoWeights &lobatto() { static LobattoWeights lw; return lw; }

// cos(j*k*pi/N) for the seven Chebyshev moments.
struct CosTable {
    real v[7 * kSamples];
    CosTable() {
        for (int k = 0; k < 7; k++)
            for (int j = 0; j < kSamples; j++)
                v[k * kSamples + j] = std::cos(j * k * kPi / kSamples);
    }
};
const CosTable &costab() { static CosTable ct; return ct; }

// Optimal nodal first derivatives: a tridiagonal least-squares system over the
// Hermite cardinal functions.  With fixed ends the end rows pin fp(a), fp(b).
void nodal_derivatives(const Interpoland &I, int n, const real *x, real *fp,
                       bool fixed_ends, real fpa, real fpb) {
    const real cwl1[4] = {0.25, -0.25, -0.25, 0.25};
    const real cwr1[4] = {-0.25, -0.25, 0.25, 0.25};
    const real wl0wl1 = 0.1125317885884428;
    const real wl1wl1 = 0.03215579530433858;
    const real wl0wr1 = -0.04823369227661384;
    const real wl1wr1 = -0.02143719641629633;
    const real wr0wr1 = -0.1125317885884429;
    const real wr1wr1 = 0.03215579530433859;
    const real wl1wr0 = 0.04823369227661384;
    const LobattoWeights &L = lobatto();

    std::vector<real> fx(n + 1, 0.0f), hx(n, 0.0f);
    std::vector<real> d0(n + 1, 0.0f), d1(n + 1, 0.0f), d2(n + 1, 0.0f), rhs(n + 1, 0.0f);
    std::vector<real> vl(n, 0.0f), vr(n, 0.0f);

    for (int i = 0; i <= n; i++) fx[i] = I.f(x[i]);
    for (int i = 0; i < n; i++) hx[i] = x[i + 1] - x[i];

    for (int i = 0; i < n; i++) {
        real m = 0.5 * (x[i] + x[i + 1]);
        real h = 0.5 * (x[i + 1] - x[i]);
        real sl = 0.0, sr = 0.0;
        for (int k = 1; k < kSamples - 1; k++) {
            real y = I.f(m + h * L.xi[k]);
            const real t = L.xi[k];
            sl += L.w[k] * (y * (cwl1[0] + t * (cwl1[1] + t * (cwl1[2] + t * cwl1[3]))));
            sr += L.w[k] * (y * (cwr1[0] + t * (cwr1[1] + t * (cwr1[2] + t * cwr1[3]))));
        }
        vl[i] = sl / (kSamples - 2);
        vr[i] = sr / (kSamples - 2);
    }

    if (fixed_ends) {
        d1[0] = 1.0; d2[0] = 0.0; rhs[0] = fpa;
    } else {
        d1[0] = wl1wl1 * hx[0];
        d2[0] = wl1wr1 * hx[0];
        rhs[0] = 2 * (vl[0] - fx[0] * wl0wl1 - fx[1] * wl1wr0);
    }
    for (int i = 1; i < n; i++) {
        d0[i] = wl1wr1 * hx[i - 1];
        d1[i] = wr1wr1 * hx[i - 1] + wl1wl1 * hx[i];
        d2[i] = wl1wr1 * hx[i];
        rhs[i] = 2 * (vr[i - 1] - fx[i - 1] * wl0wr1 - fx[i] * wr0wr1) +
                 2 * (vl[i] - fx[i] * wl0wl1 - fx[i + 1] * wl1wr0);
    }
    if (fixed_ends) {
        d0[n] = 0.0; d1[n] = 1.0; rhs[n] = fpb;
    } else {
        d0[n] = wl1wr1 * hx[n - 1];
        d1[n] = wr1wr1 * hx[n - 1];
        rhs[n] = 2 * (vr[n - 1] - fx[n - 1] * wl0wr1 - fx[n] * wr0wr1);
    }

    // Thomas algorithm.
    for (int i = 1; i <= n; i++) {
        real m = d0[i] / d1[i - 1];
        d1[i] = d1[i] - m * d2[i - 1];
        rhs[i] = rhs[i] - m * rhs[i - 1];
    }
    fp[n] = rhs[n] / d1[n];
    for (int i = n - 1; i >= 0; i--) fp[i] = (rhs[i] - d2[i] * fp[i + 1]) / d1[i];
}

// Quintic coefficients of every interval between nodes xi[0..n]; writes interval i at
// c[i*kChunk] and returns the largest locally-relative interpolation error.
real interval_coefficients(const Interpoland &I, const real *xi, int n, real *c) {
    const CosTable &C = costab();
    std::vector<real> fix(n + 1, 0.0f), fpx(n + 1, 0.0f);
    real fx[kSamples];
    real phi[7], cee[6];

    for (int k = 0; k <= n; k++) fix[k] = I.f(xi[k]);
    if (I.fp)
        nodal_derivatives(I, n, xi, fpx.data(), true, I.fp(xi[0]), I.fp(xi[n]));
    else
        nodal_derivatives(I, n, xi, fpx.data(), false, 0.0f, 0.0f);

    real err = 0.0;
    for (int i = 0; i < n; i++) {
        real *ci = c + i * kChunk;
        real m = (xi[i] + xi[i + 1]) / 2;
        real h = (xi[i + 1] - xi[i]) / 2;
        real fa = fix[i], fb = fix[i + 1];
        real dfa = fpx[i] * h, dfb = fpx[i + 1] * h;

        // Chebyshev moments of f over the interval.
        for (int k = 0; k < kSamples; k++) fx[k] = I.f(m + h * std::cos(k * kPi / kSamples));
        for (int j = 0; j < 7; j++) {
            phi[j] = (fa + (1 - 2 * (j % 2)) * fb) / 2;
            for (int k = 1; k < kSamples; k++) phi[j] += fx[k] * C.v[j * kSamples + k];
            phi[j] *= 2.0 / kSamples;
        }

        // Cubic Hermite part, then the 4th and 5th order corrections.
        cee[0] = (4 * (fa + fb) + dfa - dfb) / 4;
        cee[1] = -(9 * (fa - fb) + dfa + dfb) / 16;
        cee[2] = (dfb - dfa) / 8;
        cee[3] = (fa - fb + dfa + dfb) / 16;
        cee[4] = 0.0;
        cee[5] = 0.0;
        real w = (6 * (cee[0] - phi[0]) - 4 * (cee[2] - phi[2]) - phi[4]) / (36 + 16 + 1);
        cee[0] += -6 * w;
        cee[2] += 4 * w;
        cee[4] = -w;
        w = (2 * (cee[1] - phi[1]) - 3 * (cee[3] - phi[3]) - phi[5]) / (4 + 9 + 1);
        cee[1] += -2 * w;
        cee[3] += 3 * w;
        cee[5] = -w;

        // Chebyshev -> monomials on [-1,1]; highest power first from slot 2.
        ci[7] = cee[0] / 2 - cee[2] + cee[4];
        ci[6] = cee[1] - 3 * cee[3] + 5 * cee[5];
        ci[5] = 2 * cee[2] - 8 * cee[4];
        ci[4] = 4 * cee[3] - 20 * cee[5];
        ci[3] = 8 * cee[4];
        ci[2] = 16 * cee[5];
        ci[1] = 1.0 / h;
        ci[0] = m;

        real maxf = 0.0, err_loc = 0.0;
        for (int k = 1; k < kSamples; k++) {
            maxf = std::fmax(std::fabs(fx[k]), maxf);
            real t = C.v[kSamples + k];
            real e = std::fabs(fx[k] - ci[7] -
                               t * (ci[6] + t * (ci[5] + t * (ci[4] + t * (ci[3] + t * ci[2])))));
            err_loc = std::fmax(e, err_loc);
        }
        err_loc /= std::fmax((double)maxf, 1.0);
        err = std::fmax(err_loc, err);
    }
    return err;
}

// Golden-section search for the node-density parameter that equalises the sixth
// derivative bound across the domain.
real node_alpha(const Interpoland &I, real a, real b) {
    real xi[kSamples], fx[kSamples];
    real maxf = 0.0;
    const real golden = 2.0 / (1 + std::sqrt(5));
    for (int i = 0; i < kSamples; i++) {
        xi[i] = ((real)i + 1) / (kSamples + 1);
        fx[i] = I.f6p(a + (b - a) * xi[i]);
        maxf = std::fmax(maxf, std::fabs(fx[i]));
    }
    if (maxf == 0.0) return 1.0;

    auto bound = [&](real al) {
        real m = 0.0;
        for (int j = 0; j < kSamples; j++) {
            real t = std::fabs(std::pow(al + 2 * (1 - al) * xi[j], -6) * fx[j]);
            if (t > m) m = t;
        }
        return m;
    };
    real al[4], fa[4];
    al[0] = 0; al[3] = 2;
    al[1] = al[3] - 2 * golden;
    al[2] = al[0] + 2 * golden;
    for (int i = 0; i < 4; i++) fa[i] = bound(al[i]);
    while (al[3] - al[0] > 1.0e-4) {
        int i;
        if (fa[1] < fa[2]) {
            al[3] = al[2]; fa[3] = fa[2];
            al[2] = al[1]; fa[2] = fa[1];
            al[1] = al[3] - (al[3] - al[0]) * golden;
            i = 1;
        } else {
            al[0] = al[1]; fa[0] = fa[1];
            al[1] = al[2]; fa[1] = fa[2];
            al[2] = al[0] + (al[3] - al[0]) * golden;
            i = 2;
        }
        fa[i] = bound(al[i]);
    }
    return (al[0] + al[3]) / 2;
}

// Nodes xi[0..n] of the transform t(x) = alpha0 + x*(alpha1 + x*alpha2), placed at
// t = i/n by Newton iteration.
// The reference iterates without a bound; a table whose iteration has not converged
// after 100,000 steps is refused instead of hanging the host.
bool place_nodes(const real *alpha, real a, real b, int n, real *xi) {
    const real mtol = 10 * FLT_EPSILON;
    xi[0] = a; xi[n] = b;
    for (int i = 1; i < n; i++) {
        xi[i] = a + (b - a) * i / n;
        for (int it = 0;; it++) {
            real e = i - n * (alpha[0] + xi[i] * (alpha[1] + xi[i] * alpha[2]));
            xi[i] += e / (n * (alpha[1] + 2 * xi[i] * alpha[2]));
            if (std::fabs((double)e) < n * mtol) break;
            if (it > 100000) return false;
        }
    }
    return true;
}

struct Table {
    int n = 0;
    std::vector<real> c;   // (n+1)*kChunk; slot 0 is the continuation interval
};

// One interpolation with n intervals: returns its error and fills t.
real build_with(const Interpoland &I, const real *alpha, real a, real b, int n, Table &t) {
    std::vector<real> xi(n + 1);
    t.n = n;
    t.c.assign((size_t)(n + 1) * kChunk, 0.0f);
    if (!place_nodes(alpha, a, b, n, xi.data())) {
        t.n = -1;
        return INFINITY;
    }
    return interval_coefficients(I, xi.data(), n, t.c.data() + kChunk);
}

// Slot 0: quadratic continuation of interval 1 to the left of a.
void continue_first_interval(real *c, real a) {
    c[0] = a; c[1] = 1.0 / a;
    real coeffs[kDegree], eff[kDegree];
    for (int k = 0; k < kDegree; k++) {
        coeffs[k] = c[2 * kChunk - 1 - k];
        eff[k] = 0.0;
    }
    for (int i = 0; i < kDegree; i++)
        for (int k = kDegree - 1; k >= i; k--) {
            eff[i] = coeffs[k] + (-1.0) * eff[i];
            coeffs[k] *= (k - i) * c[kChunk + 1] * a;
        }
    c[kChunk - 1] = eff[0];
    c[kChunk - 2] = eff[1];
    c[kChunk - 3] = 0.5 * eff[2];
    for (int k = 3; k <= kDegree; k++) c[kChunk - 1 - k] = 0.0;
}

struct Built {
    int status = TFG_OK;
    real alpha[4] = {0, 0, 0, 0};
    real a = 0, b = 0;
    Table table;
};

Built init_table(const Interpoland &I, real a, real b, real tol) {
    Built out;
    out.a = a; out.b = b;
    b = (real)(b + std::fabs((double)b) * std::sqrt((double)FLT_EPSILON));
    a = (real)(a - std::fabs((double)a) * std::sqrt((double)FLT_EPSILON));

    real al = node_alpha(I, a, b);
    real *A = out.alpha;
    real w = 1.0 / (a - b);
    w *= w;
    A[0] = a * a * w - al * b * a * w;
    A[1] = -2 * a * w + al * (a + b) * w;
    A[2] = w - al * w;
    A[3] = 0.0;
    w = (real)(2 * FLT_EPSILON * (std::fabs((double)A[0]) + std::fabs((double)A[1]) + std::fabs((double)A[2])));
    A[0] -= w * a / (a - b);
    A[1] += w / (a - b);

    int l = kIvalsA, r = kIvalsB;
    Table tl, tr;
    real err_l = build_with(I, A, a, b, l, tl);
    if (tl.n < 0) { out.status = TFG_E_INVAL; return out; }
    Table *chosen = nullptr;
    if (err_l < tol) {
        chosen = &tl;
    } else {
        // Double the right bracket until it meets the tolerance.
        for (;;) {
            real err_r = build_with(I, A, a, b, r, tr);
            if (tr.n < 0) { out.status = TFG_E_INVAL; return out; }
            if (err_r < tol) break;
            if (2 * r > kIvalsMax) { out.status = TFG_E_OVERFLOW; return out; }
            l = r; tl = tr;
            r *= 2;
        }
        // Bisect for the smallest interval count below tolerance.
        while (r - l > 1) {
            int m = 0.5 * (r + l);
            Table tm;
            real err_m = build_with(I, A, a, b, m, tm);
            if (tm.n < 0) { out.status = TFG_E_INVAL; return out; }
            if (err_m > tol) { l = m; tl = std::move(tm); }
            else { r = m; tr = std::move(tm); }
        }
        chosen = &tr;
    }
    out.table = std::move(*chosen);
    int n = out.table.n;
    A[0] *= n; A[1] *= n; A[2] *= n;
    A[0] += 1.0;
    continue_first_interval(out.table.c.data(), a);
    return out;
}

// Library-owned potential: the public struct plus its table storage.
struct OwnedPotential {
    tfg_potential pub;
    std::vector<float> c;
};

int publish(const Built &b, uint32_t flags, float r0_plusone, tfg_potential **out) {
    if (b.status != TFG_OK) return b.status;
    OwnedPotential *op = new (std::nothrow) OwnedPotential();
    if (!op) return TFG_E_OOM;
    std::memset(&op->pub, 0, sizeof(op->pub));
    op->c = b.table.c;
    op->pub.kind = TFG_POTENTIAL_KIND_POTENTIAL;
    op->pub.flags = flags;
    for (int k = 0; k < 4; k++) op->pub.alpha[k] = b.alpha[k];
    op->pub.r0_plusone = r0_plusone;
    op->pub.a = b.a;
    op->pub.b = b.b;
    op->pub.n = b.table.n;
    op->pub.c = op->c.data();
    *out = &op->pub;
    return TFG_OK;
}

real powr(real base, real e) { return std::pow(base, e); }   // the reference's Power()

}  // namespace

extern "C" {

TFG_API int tfg_potential_morse(float d, float a, float r0, float min, float max, float tol,
                                int shifted, tfg_potential **out) {
    if (!out || !(max > min) || tol <= 0) return TFG_E_INVAL;
    const real E = (real)M_E;
    Interpoland I;
    if (shifted) {
        I.f = [=](real r) { return d * (powr(E, -2 * a * (-1 + r)) - 2 / powr(E, a * (-1 + r))); };
        I.fp = [=](real r) {
            return d * ((-2 * a) / powr(E, 2 * a * (-1 + r)) + (2 * a) / powr(E, a * (-1 + r)));
        };
        I.f6p = [=](real r) {
            return d * ((64 * powr(a, 6)) / powr(E, 2 * a * (-1 + r)) -
                        (2 * powr(a, 6)) / powr(E, a * (-1 + r)));
        };
        Built b = init_table(I, min + 1, max + 1, tol);
        return publish(b, TFG_POTENTIAL_R2 | TFG_POTENTIAL_SHIFTED, r0 + 1, out);
    }
    I.f = [=](real r) { return d * (powr(E, 2 * a * (r0 - r)) - 2 * powr(E, a * (r0 - r))); };
    I.fp = [=](real r) { return -2 * a * d * (powr(E, 2 * a * (r0 - r)) - powr(E, a * (r0 - r))); };
    I.f6p = [=](real r) {
        return 2 * powr(a, 6) * d * (32 * powr(E, 2 * a * (r0 - r)) - powr(E, a * (r0 - r)));
    };
    Built b = init_table(I, min, max, tol);
    return publish(b, TFG_POTENTIAL_R2, r0 + 1, out);
}

TFG_API int tfg_potential_lennard_jones_12_6(float min, float max, float A, float B, float tol,
                                             tfg_potential **out) {
    if (!out || !(max > min) || !(min > 0)) return TFG_E_INVAL;
    if (tol <= 0) tol = 0.001 * (max - min);
    Interpoland I;
    I.f = [=](real r) {
        real ir = 1.0 / r, ir2 = ir * ir, ir6 = ir2 * ir2 * ir2, ir12 = ir6 * ir6;
        return A * ir12 - B * ir6;
    };
    I.fp = [=](real r) {
        real ir = 1.0 / r, ir2 = ir * ir, ir4 = ir2 * ir2, ir12 = ir4 * ir4 * ir4;
        return (real)(6.0 * ir * (-2.0 * A * ir12 + B * ir4 * ir2));
    };
    I.f6p = [=](real r) {
        real r2 = r * r, ir2 = 1.0 / r2, ir6 = ir2 * ir2 * ir2, ir12 = ir6 * ir6;
        return (real)(10080.0 * ir12 * (884.0 * A * ir6 - 33.0 * B));
    };
    Built b = init_table(I, min, max, tol);
    // r0_plusone keeps Potential's default 1 (tfPotential.cpp:63); LJ is not shifted.
    return publish(b, TFG_POTENTIAL_R2 | TFG_POTENTIAL_LJ126, 1.0f, out);
}

TFG_API int tfg_potential_harmonic(float k, float r0, float min, float max, float tol,
                                   tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    float range = r0;
    if (min < 0) min = r0 - range;
    if (max < 0) max = r0 + range;
    if (!(max > min)) return TFG_E_INVAL;
    if (tol <= 0) tol = 0.01 * (max - min);
    Interpoland I;
    I.f = [=](real r) { return k * (r - r0) * (r - r0); };
    I.fp = [=](real r) { return (real)(2.0 * k * (r - r0)); };
    I.f6p = [](real) { return (real)0; };
    Built b = init_table(I, min, max, tol);
    // potential_create_harmonic sets flags = POTENTIAL_HARMONIC & POTENTIAL_R2 == 0
    // (tfPotential.cpp:374): no shift, no scaling.
    return publish(b, TFG_POTENTIAL_HARMONIC & TFG_POTENTIAL_R2, r0 + 1, out);
}

TFG_API int tfg_potential_harmonic_angle(float k, float theta0, float min, float max, float tol,
                                         tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    // The wrapper's defaults are double literals, so its range and default tolerance are
    // doubles (tfPotential.cpp:2995-2997) until they are passed on as FPTYPE.
    const double lo = min < 0 ? 0.0 : (double)min;
    const double hi = max < 0 ? M_PI : (double)max;
    if (tol <= 0) tol = 0.005 * (hi - lo);
    real a = lo, b = hi;
    if (a < 0.0) a = 0.0;
    if (b > M_PI) b = M_PI;
    real left = std::cos((double)b), right = std::cos((double)a);
    Interpoland I;
    I.f = [=](real r) {
        r = std::fmin(1.0, std::fmax(-1.0, (double)r));
        real theta = std::acos((double)r);
        return k * (theta - theta0) * (theta - theta0);
    };
    I.f6p = [](real) { return (real)0; };
    Built bt = init_table(I, left, right, tol);
    return publish(bt, TFG_POTENTIAL_ANGLE | TFG_POTENTIAL_HARMONIC, 1.0f, out);
}

TFG_API int tfg_potential_dpd(float alpha, float gamma, float sigma, float cutoff, int shifted,
                              tfg_potential **out) {
    if (!out || !(cutoff > 0)) return TFG_E_INVAL;
    OwnedPotential *op = new (std::nothrow) OwnedPotential();
    if (!op) return TFG_E_OOM;
    std::memset(&op->pub, 0, sizeof(op->pub));
    op->pub.kind = TFG_POTENTIAL_KIND_DPD;
    op->pub.flags = shifted ? TFG_POTENTIAL_SHIFTED : 0u;
    // Potential's defaults for the fields DPD leaves alone (tfPotential.cpp:59-81): n = 1,
    // r0_plusone = 1; no table.
    op->pub.n = 1;
    op->pub.r0_plusone = 1.0f;
    op->pub.a = std::sqrt(FLT_EPSILON);
    op->pub.b = cutoff;
    op->pub.dpd_alpha = alpha;
    op->pub.dpd_gamma = gamma;
    op->pub.dpd_sigma = sigma;
    *out = &op->pub;
    return TFG_OK;
}

TFG_API void tfg_potential_free(tfg_potential *p) {
    if (!p) return;
    // pub is the first member of OwnedPotential.
    delete reinterpret_cast<OwnedPotential *>(p);
}

TFG_API int tfg_potential_eval(const tfg_potential *p, float ri, float rj, float r2,
                               float *e, float *f) {
    if (!p || !p->c || p->kind != TFG_POTENTIAL_KIND_POTENTIAL) return 0;
    const real eps = FLT_EPSILON;
    real r = std::sqrt(r2);
    real ro = r < eps ? eps : r;
    if (p->flags & TFG_POTENTIAL_SCALED) r = r / (ri + rj);
    else if (p->flags & TFG_POTENTIAL_SHIFTED) r = r - (ri + rj) + p->r0_plusone;
    r = r < p->a ? p->a : r;
    unsigned ind = std::max(0.0f, p->alpha[0] + r * (p->alpha[1] + r * p->alpha[2]));
    if (r > p->b || ind > (unsigned)p->n) return 0;
    const real *c = p->c + ind * kChunk;
    real x = (r - c[0]) * c[1];
    real ee = c[2] * x + c[3], eff = c[2];
    for (int k = 4; k < kChunk; k++) {
        eff = eff * x + ee;
        ee = ee * x + c[k];
    }
    if (e) *e = ee;
    if (f) *f = eff * c[1] / ro;
    return 1;
}

}  // extern "C"
