// Oracle-side construction of Tissue Forge's tabulated potentials.
//
// TEST INFRASTRUCTURE ONLY.  This is the checker's own restatement of the reference's
// table builder, written from source/mdcore/src/tfPotential.cpp and independent of the
// product library: the oracle engine builds its potentials here, and a CPU test
// compares every table word of the product's builder against these.
//
// Arithmetic types follow the reference's single-precision build (FPTYPE = float,
// mdcore_config.h.in:40-53) word for word, including its C++ overload resolution:
// tfPotential.cpp includes <cmath> and never <math.h> (no header of the reference tree
// includes <math.h> or brings std:: names into the global namespace), so an unqualified
// fabs/sqrt/cos/acos/fmax/pow on a float argument calls the C library's DOUBLE function
// and the result is rounded back only when stored into an FPTYPE.  Explicitly qualified
// std:: calls on floats (Power(), tfPotential.cpp:1177-1180; DPDPotential's
// std::sqrt, tfDPDPotential.cpp:37) use the float overloads.  Compiled with
// -ffp-contract=off: no FMA contraction, as the reference's x86 build (-mavx, no -mfma).
//
// Restated steps (file tfPotential.cpp unless noted):
//   potential_init          :1396-1634  domain stretch, transform, node placement,
//                                       interval-count doubling and bisection,
//                                       linear continuation of interval 0
//   potential_getfp         :1650-1731  optimal first derivatives (free ends)
//   potential_getfp_fixend  :1734-1815  optimal first derivatives (given end slopes)
//   potential_getcoeffs     :1839-1961  Chebyshev moments -> quintic monomials, error
//   potential_getalpha      :1977-2040  golden-section search of the node density
//   Morse                   :2188-2283 (Power :1177-1180), wrapper :3068-3084
//   Lennard-Jones 12-6      :192-245, :1057-1109, wrapper :2741-2751
//   harmonic                :343-401, wrapper :2961-2975
//   harmonic angle          :550-626, wrapper :2991-3003
//   DPD                     tfDPDPotential.cpp:32-43, wrapper tfPotential.cpp:3128-3142
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "tfg.h"

namespace {

typedef float F;  // FPTYPE

constexpr int kDegree = 5;                 // potential_degree     tfPotential.h:39
constexpr int kChunk = kDegree + 3;        // potential_chunk      :40
constexpr int kIvalsA = 1;                 // potential_ivalsa     :41
constexpr int kIvalsB = 10;                // potential_ivalsb     :42
constexpr int kN = 100;                    // potential_N          :43
constexpr int kIvalsMax = 3048;            // potential_ivalsmax   :45
constexpr double kPi = 3.14159265358979323846;   // M_PI
constexpr double kE = 2.7182818284590452354;     // M_E

// The C library's double functions, named for what the reference's unqualified calls on
// float arguments resolve to.
inline double c_fabs(double x) { return ::fabs(x); }
inline double c_sqrt(double x) { return ::sqrt(x); }
inline double c_cos(double x) { return ::cos(x); }
inline double c_acos(double x) { return ::acos(x); }
inline double c_fmax(double x, double y) { return ::fmax(x, y); }
inline double c_fmin(double x, double y) { return ::fmin(x, y); }
inline double c_pow(double x, double y) { return ::pow(x, y); }
// Power(FPTYPE, FPTYPE) = std::pow on two floats: the float overload.
inline F Power(F base, F ex) { return std::pow(base, ex); }

// The function being tabulated: value, first derivative (optional) and sixth derivative.
struct Interpoland {
    virtual ~Interpoland() {}
    virtual F f(F r) const = 0;
    virtual bool has_fp() const { return true; }
    virtual F fp(F r) const = 0;
    virtual F f6p(F r) const = 0;
};

// ---- potential_getalpha (:1977-2040) ----
F getalpha(const Interpoland &I, F a, F b) {
    F xi[kN], fx[kN];
    F alpha[4], fa[4], maxf = 0.0;
    const F golden = (F)(2.0 / (1 + c_sqrt(5)));
    for (int i = 0; i < kN; i++) {
        xi[i] = ((F)i + 1) / (kN + 1);
        fx[i] = I.f6p(a + (b - a) * xi[i]);
        maxf = (F)c_fmax(maxf, c_fabs(fx[i]));
    }
    if (maxf == 0.0) return 1.0;
    auto worst = [&](F al) {
        F m = 0.0;
        for (int j = 0; j < kN; j++) {
            F t = (F)c_fabs(c_pow(al + 2 * (1 - al) * xi[j], -6) * fx[j]);
            if (t > m) m = t;
        }
        return m;
    };
    alpha[0] = 0;
    alpha[3] = 2;
    alpha[1] = alpha[3] - 2 * golden;
    alpha[2] = alpha[0] + 2 * golden;
    for (int i = 0; i < 4; i++) fa[i] = worst(alpha[i]);
    while (alpha[3] - alpha[0] > 1.0e-4) {
        int i;
        if (fa[1] < fa[2]) {
            alpha[3] = alpha[2]; fa[3] = fa[2];
            alpha[2] = alpha[1]; fa[2] = fa[1];
            alpha[1] = alpha[3] - (alpha[3] - alpha[0]) * golden;
            i = 1;
        } else {
            alpha[0] = alpha[1]; fa[0] = fa[1];
            alpha[1] = alpha[2]; fa[1] = fa[2];
            alpha[2] = alpha[0] + (alpha[3] - alpha[0]) * golden;
            i = 2;
        }
        fa[i] = worst(alpha[i]);
    }
    return (alpha[0] + alpha[3]) / 2;
}

// Cosine-weighted sample points of potential_getfp (:1662-1674): xi = cos(k pi/(N-1)),
// w = 1/sqrt(1 - xi^2), zero weight at the two ends.
struct FpWeights {
    F xi[kN], w[kN];
    FpWeights() {
        for (int k = 1; k < kN - 1; k++) {
            xi[k] = (F)c_cos(k * kPi / (kN - 1));
            w[k] = (F)(1.0 / c_sqrt(1.0 - xi[k] * xi[k]));
        }
        xi[0] = 1.0;
        xi[kN - 1] = -1.0;
        w[0] = 0.0;
        w[kN - 1] = 0.0;
    }
};
const FpWeights &fp_weights() {
    static const FpWeights W;
    return W;
}

// ---- potential_getfp (:1650-1731) and potential_getfp_fixend (:1734-1815) ----
// First derivatives at the nodes x[0..n] that minimise the interpolation error: a
// tridiagonal system from the projections of f on the cubic cardinal functions.  With
// fixed ends the first and last rows are fp = fpa and fp = fpb.
void getfp(const Interpoland &I, int n, const F *x, F *fp, bool fixend, F fpa, F fpb) {
    const FpWeights &W = fp_weights();
    std::vector<F> fx(n + 1, 0.0f), hx(n, 0.0f);
    std::vector<F> d0(n + 1, 0.0f), d1(n + 1, 0.0f), d2(n + 1, 0.0f), b(n + 1, 0.0f);
    std::vector<F> viwl1(n, 0.0f), viwr1(n, 0.0f);
    const F cwl1[4] = {0.25, -0.25, -0.25, 0.25};
    const F cwr1[4] = {-0.25, -0.25, 0.25, 0.25};
    const F wl0wl1 = 0.1125317885884428;
    const F wl1wl1 = 0.03215579530433858;
    const F wl0wr1 = -0.04823369227661384;
    const F wl1wr1 = -0.02143719641629633;
    const F wr0wr1 = -0.1125317885884429;
    const F wr1wr1 = 0.03215579530433859;
    const F wl1wr0 = 0.04823369227661384;

    for (int i = 0; i <= n; i++) fx[i] = I.f(x[i]);
    for (int i = 0; i < n; i++) hx[i] = x[i + 1] - x[i];
    for (int i = 0; i < n; i++) {
        F l = 0.0, r = 0.0;
        const F m = (F)(0.5 * (x[i] + x[i + 1]));
        const F h = (F)(0.5 * (x[i + 1] - x[i]));
        for (int k = 1; k < kN - 1; k++) {
            const F t = W.xi[k];
            const F eff = I.f(m + h * t);
            l += W.w[k] * (eff * (cwl1[0] + t * (cwl1[1] + t * (cwl1[2] + t * cwl1[3]))));
            r += W.w[k] * (eff * (cwr1[0] + t * (cwr1[1] + t * (cwr1[2] + t * cwr1[3]))));
        }
        viwl1[i] = l / (kN - 2);
        viwr1[i] = r / (kN - 2);
    }
    if (fixend) {
        d1[0] = 1.0;
        d2[0] = 0.0;
        b[0] = fpa;
    } else {
        d1[0] = wl1wl1 * hx[0];
        d2[0] = wl1wr1 * hx[0];
        b[0] = 2 * (viwl1[0] - fx[0] * wl0wl1 - fx[1] * wl1wr0);
    }
    for (int i = 1; i < n; i++) {
        d0[i] = wl1wr1 * hx[i - 1];
        d1[i] = wr1wr1 * hx[i - 1] + wl1wl1 * hx[i];
        d2[i] = wl1wr1 * hx[i];
        b[i] = 2 * (viwr1[i - 1] - fx[i - 1] * wl0wr1 - fx[i] * wr0wr1) +
               2 * (viwl1[i] - fx[i] * wl0wl1 - fx[i + 1] * wl1wr0);
    }
    if (fixend) {
        d0[n] = 0.0;
        d1[n] = 1.0;
        b[n] = fpb;
    } else {
        d0[n] = wl1wr1 * hx[n - 1];
        d1[n] = wr1wr1 * hx[n - 1];
        b[n] = 2 * (viwr1[n - 1] - fx[n - 1] * wl0wr1 - fx[n] * wr0wr1);
    }
    // Thomas algorithm, forward elimination then back substitution
    for (int i = 1; i <= n; i++) {
        const F m = d0[i] / d1[i - 1];
        d1[i] = d1[i] - m * d2[i - 1];
        b[i] = b[i] - m * b[i - 1];
    }
    fp[n] = b[n] / d1[n];
    for (int i = n - 1; i >= 0; i--) fp[i] = (b[i] - d2[i] * fp[i + 1]) / d1[i];
}

// cos(j k pi / N) for j = 0..6 moments (the static coskx table of :1855-1861).
struct ChebCos {
    F v[7 * kN];
    ChebCos() {
        for (int k = 0; k < 7; k++)
            for (int j = 0; j < kN; j++) v[k * kN + j] = (F)c_cos(j * k * kPi / kN);
    }
};
const ChebCos &cheb_cos() {
    static const ChebCos C;
    return C;
}

// ---- potential_getcoeffs (:1839-1961) ----
// Coefficients of the n intervals between the nodes xi into c[8 i .. 8 i + 7] (interval
// centre, inverse half-width, then the quintic's monomials from the highest power), and
// the largest local relative error estimate into *err.
void getcoeffs(const Interpoland &I, const F *xi, int n, F *c, F *err) {
    const ChebCos &CC = cheb_cos();
    std::vector<F> fix(n + 1, 0.0f), fpx(n + 1, 0.0f);
    F fx[kN];
    for (int k = 0; k <= n; k++) fix[k] = I.f(xi[k]);
    if (!I.has_fp())
        getfp(I, n, xi, fpx.data(), false, 0.0f, 0.0f);
    else
        getfp(I, n, xi, fpx.data(), true, I.fp(xi[0]), I.fp(xi[n]));
    *err = 0.0;
    for (int i = 0; i < n; i++) {
        F *ci = c + i * (kDegree + 3);
        const F m = (xi[i] + xi[i + 1]) / 2;
        const F h = (xi[i + 1] - xi[i]) / 2;
        const F fa = fix[i], fb = fix[i + 1];
        const F dfa = fpx[i] * h, dfb = fpx[i + 1] * h;
        F phi[7], cee[6];
        for (int k = 0; k < kN; k++) fx[k] = I.f((F)(m + h * c_cos(k * kPi / kN)));
        for (int j = 0; j < 7; j++) {
            F s = (fa + (1 - 2 * (j % 2)) * fb) / 2;
            for (int k = 1; k < kN; k++) s += fx[k] * CC.v[j * kN + k];
            phi[j] = (F)(s * (2.0 / kN));
        }
        // cubic Hermite part in Chebyshev form
        cee[0] = (4 * (fa + fb) + dfa - dfb) / 4;
        cee[1] = -(9 * (fa - fb) + dfa + dfb) / 16;
        cee[2] = (dfb - dfa) / 8;
        cee[3] = (fa - fb + dfa + dfb) / 16;
        cee[4] = 0.0;
        cee[5] = 0.0;
        // 4th- and 5th-order corrections that keep the end values and slopes
        F w = (6 * (cee[0] - phi[0]) - 4 * (cee[2] - phi[2]) - phi[4]) / (36 + 16 + 1);
        cee[0] += -6 * w;
        cee[2] += 4 * w;
        cee[4] = -w;
        w = (2 * (cee[1] - phi[1]) - 3 * (cee[3] - phi[3]) - phi[5]) / (4 + 9 + 1);
        cee[1] += -2 * w;
        cee[3] += 3 * w;
        cee[5] = -w;
        // Chebyshev -> monomials on [-1, 1]
        ci[7] = cee[0] / 2 - cee[2] + cee[4];
        ci[6] = cee[1] - 3 * cee[3] + 5 * cee[5];
        ci[5] = 2 * cee[2] - 8 * cee[4];
        ci[4] = 4 * cee[3] - 20 * cee[5];
        ci[3] = 8 * cee[4];
        ci[2] = 16 * cee[5];
        ci[1] = (F)(1.0 / h);
        ci[0] = m;
        F maxf = 0.0, err_loc = 0.0;
        for (int k = 1; k < kN; k++) {
            maxf = (F)c_fmax(c_fabs(fx[k]), maxf);
            const F x = CC.v[kN + k];
            const F e = (F)c_fabs(fx[k] - ci[7] - x * (ci[6] + x * (ci[5] + x * (ci[4] + x * (ci[3] + x * ci[2])))));
            err_loc = (F)c_fmax(e, err_loc);
        }
        err_loc = (F)(err_loc / c_fmax(maxf, 1.0));
        *err = (F)c_fmax(err_loc, *err);
    }
}

// ---- potential_init (:1396-1634) ----
// Node placement of :1457-1465: Newton iteration on the transformed index
// i = l (alpha0 + x (alpha1 + x alpha2)).  The reference loops until convergence; the
// oracle stops after a generous bound and reports a failure instead of hanging.
bool place_nodes(int l, F a, F b, const F *A, F *xi) {
    const F mtol = 10 * FLT_EPSILON;
    xi[0] = a;
    xi[l] = b;
    for (int i = 1; i < l; i++) {
        xi[i] = a + (b - a) * i / l;
        int it = 0;
        while (true) {
            const F e = i - l * (A[0] + xi[i] * (A[1] + xi[i] * A[2]));
            xi[i] += e / (l * (A[1] + 2 * xi[i] * A[2]));
            if (c_fabs(e) < l * mtol) break;
            if (++it > 100000) return false;
        }
    }
    return true;
}

struct Table {
    int n = 0;
    std::vector<F> c;   // (n + 1) * kChunk
    std::vector<F> xi;  // n + 1 nodes
    F err = 0;
};

bool interpolate(const Interpoland &I, int n, F a, F b, const F *A, Table &t) {
    t.n = n;
    t.xi.assign(n + 1, 0.0f);
    t.c.assign((size_t)(n + 1) * kChunk, 0.0f);
    if (!place_nodes(n, a, b, A, t.xi.data())) return false;
    getcoeffs(I, t.xi.data(), n, t.c.data() + kChunk, &t.err);
    return true;
}

// Interval 0 (r below the first node) as a linear continuation of interval 1
// (:1609-1624): c[0] = a, c[1] = 1/a, the value and slope of interval 1 at its left end
// rewritten in interval 0's variable.
void linear_first_interval(F *c, F a) {
    c[0] = a;
    c[1] = (F)(1.0 / a);
    F coeffs[kDegree], eff[kDegree];
    for (int k = 0; k < kDegree; k++) {
        coeffs[k] = c[2 * kChunk - 1 - k];
        eff[k] = 0.0;
    }
    for (int i = 0; i < kDegree; i++)
        for (int k = kDegree - 1; k >= i; k--) {
            eff[i] = (F)(coeffs[k] + (-1.0) * eff[i]);
            coeffs[k] *= (k - i) * c[kChunk + 1] * a;
        }
    c[kChunk - 1] = eff[0];
    c[kChunk - 2] = eff[1];
    c[kChunk - 3] = (F)(0.5 * eff[2]);
    for (int k = 3; k <= kDegree; k++) c[kChunk - 1 - k] = 0.0;
}

struct OraclePot {
    tfg_potential pub;   // first member: the public pointer is the object's address
    std::vector<F> table;
};

OraclePot *new_pot() {
    OraclePot *op = new OraclePot();
    tfg_potential &p = op->pub;
    // Potential::Potential defaults (tfPotential.cpp:59-81)
    p.kind = TFG_POTENTIAL_KIND_POTENTIAL;
    p.flags = 0;
    for (int k = 0; k < 4; k++) p.alpha[k] = 0.0f;
    p.r0_plusone = 1.0f;
    p.a = 0.0f;
    p.b = FLT_MAX;
    p.n = 1;
    p.c = nullptr;
    p.dpd_alpha = p.dpd_gamma = p.dpd_sigma = 0.0f;
    return op;
}

int potential_init(OraclePot *op, const Interpoland &I, F a, F b, F tol) {
    if (!(a < b) || !(tol > 0)) return TFG_E_INVAL;
    tfg_potential &p = op->pub;
    p.a = a;
    p.b = b;
    // stretch the domain slightly against rounding in the index computation
    b = (F)(b + c_fabs(b) * c_sqrt(FLT_EPSILON));
    a = (F)(a - c_fabs(a) * c_sqrt(FLT_EPSILON));
    const F alpha = getalpha(I, a, b);
    // interval transform
    F A[4];
    F w = (F)(1.0 / (a - b));
    w *= w;
    A[0] = a * a * w - alpha * b * a * w;
    A[1] = -2 * a * w + alpha * (a + b) * w;
    A[2] = w - alpha * w;
    A[3] = 0.0;
    // correct the transform to the right
    w = (F)((2 * FLT_EPSILON) * (c_fabs(A[0]) + c_fabs(A[1]) + c_fabs(A[2])));
    A[0] -= w * a / (a - b);
    A[1] += w / (a - b);

    int l = kIvalsA, r = kIvalsB;
    Table tl, tr;
    if (!interpolate(I, l, a, b, A, tl)) return TFG_E_INVAL;
    Table *best = nullptr;
    if (tl.err < tol) {
        best = &tl;
    } else {
        // double r until it meets the tolerance
        while (true) {
            if (!interpolate(I, r, a, b, A, tr)) return TFG_E_INVAL;
            if (tr.err < tol) break;
            if (2 * r > kIvalsMax) return TFG_E_INVAL;  // too many intervals
            l = r;
            tl = tr;
            r *= 2;
        }
        // bisect between the last failing and the first passing count
        while (r - l > 1) {
            const int m = (int)(0.5 * (r + l));
            Table tm;
            if (!interpolate(I, m, a, b, A, tm)) return TFG_E_INVAL;
            if (tm.err > tol) {
                l = m;
                tl = tm;
            } else {
                r = m;
                tr = tm;
            }
        }
        best = &tr;
    }
    p.n = best->n;
    p.alpha[0] = A[0] * p.n;
    p.alpha[1] = A[1] * p.n;
    p.alpha[2] = A[2] * p.n;
    p.alpha[3] = A[3];
    p.alpha[0] = (F)(p.alpha[0] + 1.0);
    op->table = best->c;
    linear_first_interval(op->table.data(), a);
    p.c = op->table.data();
    return TFG_OK;
}

// ---- interpolands ----
// Morse (:2188-2244): the factory keeps its parameters in file statics; here they are
// members.  Power() is the float std::pow.
struct Morse : Interpoland {
    F d, a, r0;
    F f(F r) const override { return d * (Power(kE, 2 * a * (r0 - r)) - 2 * Power(kE, a * (r0 - r))); }
    F fp(F r) const override { return -2 * a * d * (Power(kE, 2 * a * (r0 - r)) - Power(kE, a * (r0 - r))); }
    F f6p(F r) const override {
        return 2 * Power(a, 6) * d * (32 * Power(kE, 2 * a * (r0 - r)) - Power(kE, a * (r0 - r)));
    }
};
struct MorseShifted : Interpoland {
    F d, a;
    F f(F r) const override { return d * (Power(kE, -2 * a * (-1 + r)) - 2 / Power(kE, a * (-1 + r))); }
    F fp(F r) const override {
        return d * ((-2 * a) / Power(kE, 2 * a * (-1 + r)) + (2 * a) / Power(kE, a * (-1 + r)));
    }
    F f6p(F r) const override {
        return d * ((64 * Power(a, 6)) / Power(kE, 2 * a * (-1 + r)) - (2 * Power(a, 6)) / Power(kE, a * (-1 + r)));
    }
};
// Lennard-Jones 12-6 (potential_LJ126, _p, _6p :192-245)
struct LJ126 : Interpoland {
    F A, B;
    F f(F r) const override {
        const F ir = (F)(1.0 / r), ir2 = ir * ir, ir6 = ir2 * ir2 * ir2, ir12 = ir6 * ir6;
        return A * ir12 - B * ir6;
    }
    F fp(F r) const override {
        const F ir = (F)(1.0 / r), ir2 = ir * ir, ir4 = ir2 * ir2, ir12 = ir4 * ir4 * ir4;
        return (F)(6.0 * ir * (-2.0 * A * ir12 + B * ir4 * ir2));
    }
    F f6p(F r) const override {
        const F r2 = r * r, ir2 = (F)(1.0 / r2), ir6 = ir2 * ir2 * ir2, ir12 = ir6 * ir6;
        return (F)(10080.0 * ir12 * (884.0 * A * ir6 - 33.0 * B));
    }
};
// harmonic bond (:343-358)
struct Harmonic : Interpoland {
    F K, r0;
    F f(F r) const override { return K * (r - r0) * (r - r0); }
    F fp(F r) const override { return (F)(2.0 * K * (r - r0)); }
    F f6p(F) const override { return 0; }
};
// harmonic angle in cos(theta) (:550-572); built without a derivative function
struct HarmonicAngle : Interpoland {
    F K, theta0;
    bool has_fp() const override { return false; }
    F f(F r) const override {
        r = (F)c_fmin(1.0, c_fmax(-1.0, r));
        const F theta = (F)c_acos(r);
        return K * (theta - theta0) * (theta - theta0);
    }
    F fp(F) const override { return 0; }
    F f6p(F) const override { return 0.0; }
};

int finish(OraclePot *op, int rc, tfg_potential **out) {
    if (rc != TFG_OK) {
        delete op;
        return rc;
    }
    *out = &op->pub;
    return TFG_OK;
}

}  // namespace

extern "C" {

// Potential::morse (:3068-3084) -> potential_create_morse (:2249-2283)
TFG_API int tfo_potential_morse(float d, float a, float r0, float min, float max, float tol, int shifted,
                                tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    OraclePot *op = new_pot();
    op->pub.flags = TFG_POTENTIAL_R2;
    op->pub.r0_plusone = r0 + 1;
    int rc;
    if (shifted) {
        MorseShifted I;
        I.d = d;
        I.a = a;
        rc = potential_init(op, I, min + 1, max + 1, tol);
        op->pub.flags |= TFG_POTENTIAL_SHIFTED;   // potential_shift (:131-134)
        op->pub.r0_plusone = r0 + 1;
    } else {
        Morse I;
        I.d = d;
        I.a = a;
        I.r0 = r0;
        rc = potential_init(op, I, min, max, tol);
    }
    return finish(op, rc, out);
}

// Potential::lennard_jones_12_6 (:2741-2751) -> potential_create_LJ126 (:1087-1109);
// tol <= 0 selects the wrapper's default 0.001 (max - min).
TFG_API int tfo_potential_lennard_jones_12_6(float min, float max, float A, float B, float tol,
                                             tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    if (!(tol > 0)) tol = (F)(0.001 * (F)(max - min));
    OraclePot *op = new_pot();
    op->pub.flags = TFG_POTENTIAL_R2 | TFG_POTENTIAL_LJ126;
    LJ126 I;
    I.A = A;
    I.B = B;
    return finish(op, potential_init(op, I, min, max, tol), out);
}

// Potential::harmonic (:2961-2975) -> potential_create_harmonic (:374-401); min < 0,
// max < 0 and tol <= 0 select the wrapper's defaults r0 - r0, r0 + r0, 0.01 (max - min).
TFG_API int tfo_potential_harmonic(float k, float r0, float min, float max, float tol, tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    const F range = r0;
    const F lo = min < 0 ? (F)(r0 - range) : min;
    const F hi = max < 0 ? (F)(r0 + range) : max;
    if (!(tol > 0)) tol = (F)(0.01 * (F)(hi - lo));
    OraclePot *op = new_pot();
    op->pub.flags = TFG_POTENTIAL_HARMONIC & TFG_POTENTIAL_R2;   // = 0, as the reference
    op->pub.r0_plusone = r0 + 1;
    Harmonic I;
    I.K = k;
    I.r0 = r0;
    return finish(op, potential_init(op, I, lo, hi, tol), out);
}

// Potential::harmonic_angle (:2991-3003) -> potential_create_harmonic_angle (:594-626);
// min < 0, max < 0 and tol <= 0 select the wrapper's defaults 0, pi, 0.005 (max - min).
// The wrapper's defaults are doubles, so its range and tolerance are formed in double.
TFG_API int tfo_potential_harmonic_angle(float k, float theta0, float min, float max, float tol,
                                         tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    const double lo = min < 0 ? 0.0 : (double)min;
    const double hi = max < 0 ? kPi : (double)max;
    if (!(tol > 0)) tol = (F)(0.005 * (hi - lo));
    F a = (F)lo, b = (F)hi;
    if (a < 0.0) a = 0.0;
    if (b > kPi) b = (F)kPi;
    const F left = (F)c_cos(b), right = (F)c_cos(a);
    OraclePot *op = new_pot();
    op->pub.flags = TFG_POTENTIAL_ANGLE | TFG_POTENTIAL_HARMONIC;
    HarmonicAngle I;
    I.K = k;
    I.theta0 = theta0;
    return finish(op, potential_init(op, I, left, right, tol), out);
}

// Potential::dpd (:3128-3142) -> DPDPotential (tfDPDPotential.cpp:32-43): no table.
TFG_API int tfo_potential_dpd(float alpha, float gamma, float sigma, float cutoff, int shifted,
                              tfg_potential **out) {
    if (!out) return TFG_E_INVAL;
    OraclePot *op = new_pot();
    op->pub.kind = TFG_POTENTIAL_KIND_DPD;
    op->pub.dpd_alpha = alpha;
    op->pub.dpd_gamma = gamma;
    op->pub.dpd_sigma = sigma;
    op->pub.a = std::sqrt(FLT_EPSILON);
    op->pub.b = cutoff;
    if (shifted) op->pub.flags |= TFG_POTENTIAL_SHIFTED;
    *out = &op->pub;
    return TFG_OK;
}

TFG_API void tfo_potential_free(tfg_potential *p) { delete reinterpret_cast<OraclePot *>(p); }

}  // extern "C"
