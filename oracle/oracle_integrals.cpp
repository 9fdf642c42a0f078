// ORACLE — test infrastructure only.
//
// CPU restatement of Quiqbox.jl v0.6.3's Gaussian-orbital integral engine, used
// exclusively by the tests, by `__graft_entry__.smoke()` and by `bench.py`'s CPU
// baseline as the checker.  The GPU product never links or calls this code.
//
// Each routine follows the reference file:line it cites, with the same
// recursions in the same order (axis-by-axis Obara–Saika with auxiliary-order
// buffers, electron transfer for two-body integrals, binomial overlap, the
// coordinate-derivative kinetic recursion), so that it is an independent check
// of the GPU kernels, which use a different (shell-based HGP / Hermite) scheme.
//
// The Boys function follows src/Integration/Engines/BoysFunction.jl.  The
// reference takes the regularised lower incomplete gamma P(a,x) from
// SpecialFunctions.jl (compat 2.5.1, not vendored); here P(a,x) is the series /
// continued-fraction pair of Press et al., "Numerical Recipes" (gser/gcf,
// §6.2), checked against mpmath at 50 digits by the tests.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double kEps = 2.220446049250313e-16;
// getAtolVal(Float64) = ceil(3eps/2, sigdigits=1) (src/Arithmetic.jl:42)
constexpr double kAtolVal = 4e-16;
// getAtolDigits(Float64) = floor(-log10(eps)) (src/Arithmetic.jl:8-16)
constexpr int kAtolDigits = 15;

// ---------------------------------------------------------------------------
// Regularised lower incomplete gamma P(a, x), a > 0, x >= 0.
double gamma_p(double a, double x) {
    if (x <= 0.0) return 0.0;
    const double gln = std::lgamma(a);
    if (x < a + 1.0) {                       // series (Numerical Recipes gser)
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 0; n < 100000; ++n) {
            ap += 1.0;
            del *= x / ap;
            sum += del;
            if (std::fabs(del) < std::fabs(sum) * 1e-17) break;
        }
        return sum * std::exp(-x + a * std::log(x) - gln);
    }
    // continued fraction for Q (Numerical Recipes gcf, modified Lentz)
    const double fpmin = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / fpmin, d = 1.0 / b, h = d;
    for (int i = 1; i < 100000; ++i) {
        const double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (std::fabs(d) < fpmin) d = fpmin;
        c = b + an / c;
        if (std::fabs(c) < fpmin) c = fpmin;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (std::fabs(del - 1.0) < 1e-17) break;
    }
    return 1.0 - std::exp(-x + a * std::log(x) - gln) * h;
}

// directComputeBoysFunc (BoysFunction.jl:7-24)
double direct_boys(double x, int n) {
    const double z = n + 0.5;
    const double p = gamma_p(z, x);
    if (p == 0.0) return 0.0;
    double res;
    if (z < 23) {
        const double part1 = std::tgamma(z) * p;
        const double part2 = std::pow(x, z);
        res = std::isinf(part2) ? std::exp(std::log(part1) - z * std::log(x)) : part1 / part2;
    } else {
        res = std::exp(std::lgamma(z) + std::log(p) - z * std::log(x));
    }
    return res / 2;
}

// initializeUpperOrder (BoysFunction.jl:27-31)
int upper_order(double x, int n) {
    const double ratio = (double(n) == x) ? double(n) : n / x;
    const int res = int(std::ceil(kAtolDigits / std::fabs(std::log10(ratio)) + n));
    return res + (res & 1);
}

// recursiveGetBoysFuncDn (BoysFunction.jl:33-40)
double boys_down(double x, int m, double val, int n) {
    const double ex = std::exp(-x);
    for (int i = m - 1; i >= n; --i) val = (2 * x * val + ex) / (2 * i + 1);
    return val;
}

}  // namespace

extern "C" {

// computeBoysFunc (BoysFunction.jl:52-64)
double qbo_boys(double x, int n) {
    if (n == 0) {
        if (x < kAtolVal) return 1.0;
        const double r = std::sqrt(x);
        return std::sqrt(kPi) * std::erf(r) / (2 * r);
    }
    if (x < kAtolVal) return 1.0 / (2 * n + 1);
    const int nup = std::min(upper_order(x, n), 6 * n);
    const double fup = direct_boys(x, nup);
    return boys_down(x, nup, fup, n);
}

// computeBoysSequence (BoysFunction.jl:67-77): out[0..n]
void qbo_boys_sequence(double x, int n, double* out) {
    out[0] = qbo_boys(x, 0);
    if (n > 0) out[n] = qbo_boys(x, n);
    for (int m = n; m >= 2; --m) out[m - 1] = boys_down(x, m, out[m], m - 1);
}

}  // extern "C"

namespace {

double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return std::round(r);
}

// computePGTOrbOverlapAxialFactor + oddFactorial (GaussianOrbitals.jl:94-97, Arithmetic.jl:101-107)
double axial_factor(double xsum, int degree) {
    double f = 1.0;
    if (degree > 0) {
        const double coeff = 1.0 / (2 * xsum);
        for (int i = 1; i <= 2 * degree - 1; i += 2) f *= i * coeff;
    }
    return std::sqrt(kPi) / std::sqrt(xsum) * f;
}

// computeGaussProd (Arithmetic.jl:110-120)
double gauss_prod(double dxML, double dxMR, int lL, int lR, int lx) {
    const int lb = std::max(-lx, lx - 2 * lR), ub = std::min(lx, 2 * lL - lx);
    double res = 0.0;
    for (int q = lb; q <= ub; q += 2) {
        const int i = (lx + q) >> 1, j = (lx - q) >> 1;
        res += binom(lL, i) * binom(lR, j) * std::pow(dxML, lL - i) * std::pow(dxMR, lR - j);
    }
    return res;
}

// computeAxialPGTOrbOverlap, adaptive form (GaussianOrbitals.jl:110-138)
double axial_overlap(double xsum, double xpos, double xML, double xMR, int iL, int iR) {
    const double dx = xMR - xML;
    if (iL == 0 && iR == 0) return axial_factor(xsum, 0) * std::exp(-xpos * dx * dx);
    if (dx == 0.0) {   // concentric: computeGaussProd(iL,iR,2j) selects 2j == iL+iR
        return ((iL + iR) % 2 == 0) ? axial_factor(xsum, (iL + iR) / 2) : 0.0;
    }
    double res = 0.0;
    for (int j = 0; j <= (iL + iR) / 2; ++j)
        res += gauss_prod(xML, xMR, iL, iR, 2 * j) * axial_factor(xsum, j);
    return res * std::exp(-xpos * dx * dx);
}

struct Prim {
    double c[3];
    double a;
    int l[3];
};

bool same_prim(const Prim& x, const Prim& y) {
    return x.a == y.a && x.c[0] == y.c[0] && x.c[1] == y.c[1] && x.c[2] == y.c[2] &&
           x.l[0] == y.l[0] && x.l[1] == y.l[1] && x.l[2] == y.l[2];
}

// GaussProductInfo (GaussianOrbitals.jl:18-37)
struct Product {
    Prim L, R;
    double cen[3];
    double xpn;
    bool sym;
};

Product make_product(const Prim& L, const Prim& R) {
    Product p{L, R, {0, 0, 0}, L.a + R.a, same_prim(L, R)};
    for (int k = 0; k < 3; ++k)
        p.cen[k] = p.sym ? L.c[k] : (L.a * L.c[k] + R.a * R.c[k]) / p.xpn;
    return p;
}

// computePGTOrbOverlap / computePGTOrbOverlap! (GaussianOrbitals.jl:147-179)
double prim_overlap(const Product& d) {
    if (d.sym) {
        double r = 1.0;
        for (int k = 0; k < 3; ++k) r *= axial_factor(2 * d.L.a, d.L.l[k]);
        return r;
    }
    const double xpos = d.L.a * d.R.a / d.xpn;
    double r = 1.0;
    for (int k = 0; k < 3; ++k)
        r *= axial_overlap(d.xpn, xpos, d.cen[k] - d.L.c[k], d.cen[k] - d.R.c[k], d.L.l[k], d.R.l[k]);
    return r;
}

// computeAxialPGTOrbCoordDiff! (GaussianOrbitals.jl:258-281)
double axial_diff(int degree, double xL, double xR, double xML, double xMR, int iL, int iR) {
    if (degree < 1) {
        const double xsum = xL + xR;
        return axial_overlap(xsum, xL * xR / xsum, xML, xMR, iL, iR);
    }
    const double dn = iR < 1 ? 0.0 : axial_diff(degree - 1, xL, xR, xML, xMR, iL, iR - 1);
    const double up = axial_diff(degree - 1, xL, xR, xML, xMR, iL, iR + 1);
    return dn * iR - up * 2 * xR;
}

// computeAxialPGTOrbCoordDiff, concentric equal-exponent form (GaussianOrbitals.jl:283-292)
double axial_diff_sym(int degree, double xpn, int iL, int iR) {
    if (degree < 1) {
        return ((iL + iR) % 2 == 0) ? axial_factor(2 * xpn, (iL + iR) / 2) : 0.0;
    }
    const double dn = iR < 1 ? 0.0 : axial_diff_sym(degree - 1, xpn, iL, iR - 1);
    const double up = axial_diff_sym(degree - 1, xpn, iL, iR + 1);
    return dn * iR - up * 2 * xpn;
}

// kinetic = Σ_axes (−½)·∂²-sandwich (Samplers.jl:81-107; GaussianOrbitals.jl:295-363,686-694)
double prim_kinetic(const Product& d) {
    double res[3] = {1.0, 1.0, 1.0};
    for (int k = 0; k < 3; ++k) {
        double diff, ovl;
        if (d.sym) {
            diff = axial_diff_sym(2, d.L.a, d.L.l[k], d.L.l[k]);
            ovl = axial_factor(2 * d.L.a, d.L.l[k]);
        } else {
            const double xML = d.cen[k] - d.L.c[k], xMR = d.cen[k] - d.R.c[k];
            diff = axial_diff(2, d.L.a, d.R.a, xML, xMR, d.L.l[k], d.R.l[k]);
            ovl = axial_overlap(d.xpn, d.L.a * d.R.a / d.xpn, xML, xMR, d.L.l[k], d.R.l[k]);
        }
        res[k] *= diff;
        for (int o = 0; o < 3; ++o)
            if (o != k) res[o] *= ovl;
    }
    return (-0.5 * res[0] + -0.5 * res[1]) + -0.5 * res[2];
}

// --- Obara–Saika Coulomb recursions (GaussianOrbitals.jl:378-663) -----------
// Buffers are 0-based; "end-k" of the reference is index (len-1-k).

// vertTransfer (GaussianOrbitals.jl:386-391)
inline double vert_transfer(double p0m1, double p1m1, double p0m2, double p1m2, int iL,
                            double xML, double xMC, double xsum, double factor) {
    const double part1 = xML * p0m1 - factor * xMC * p1m1;
    const double part2 = (iL - 1) * (p0m2 - factor * p1m2) * (1.0 / (2 * xsum));
    return part1 + part2;
}

// verticalFill! (GaussianOrbitals.jl:401-418); h has length iSum+1
void vertical_fill(double* h, int len, double xML, double xMC, double xsum, double factor) {
    const int iSum = len - 1;
    for (int n = 1; n <= iSum; ++n) {
        double b0 = h[len - 1 - n], b1 = h[len - 1 - n + 1], b2 = 0.0, b3 = 0.0;
        for (int iMax = 1; iMax <= n; ++iMax) {
            const double p0 = b0, p1 = b1;
            const double here = vert_transfer(b0, b1, b2, b3, iMax, xML, xMC, xsum, factor);
            if (iMax < n) { b0 = here; b1 = h[len - 1 - n + iMax + 1]; b2 = p0; b3 = p1; }
            h[len - 1 - n + iMax] = here;
        }
    }
}

// verticalPush! (GaussianOrbitals.jl:423-439)
void vertical_push(double* h, const double* data, int len, double xML, double xMC, double xsum,
                   double factor) {
    const int iSum = len - 1;
    double b0 = h[0], b1 = data[0], b2 = 0.0, b3 = 0.0;
    for (int i = 1; i <= iSum; ++i) {
        const double here = vert_transfer(b0, b1, b2, b3, i, xML, xMC, xsum, factor);
        h[i] = here;
        if (i < iSum) { const double a = b0, b = b1; b0 = here; b1 = data[i]; b2 = a; b3 = b; }
    }
}

// angularShift! (GaussianOrbitals.jl:446-454); operates on the last iR+1 entries of h[0..len)
double angular_shift(double* h, int len, int iR, double xLR) {
    double* seg = h + (len - 1 - iR);
    for (int y = 1; y <= iR; ++y)
        for (int x = 1; x <= iR + 1 - y; ++x) seg[x - 1] = seg[x] + xLR * seg[x - 1];
    return seg[0];
}

// computePGTOrbOneBodyRepulsion! (GaussianOrbitals.jl:478-522)
double prim_nuclear(const Product& d, const double C[3]) {
    double drLR[3], drMC[3];
    int ang[3], angSum = 0;
    for (int k = 0; k < 3; ++k) {
        drLR[k] = d.L.c[k] - d.R.c[k];
        drMC[k] = d.cen[k] - C[k];
        ang[k] = d.L.l[k] + d.R.l[k];
        angSum += ang[k];
    }
    const double xsum = d.xpn, xpos = d.L.a * d.R.a / xsum;
    double mixed = 1.0;
    for (int k = 0; k < 3; ++k) mixed *= std::exp(-xpos * drLR[k] * drLR[k]);
    const double factor = 2 * kPi * (mixed / xsum);
    const double r2 = (drMC[0] * drMC[0] + drMC[1] * drMC[1]) + drMC[2] * drMC[2];
    const int len = angSum + 1;
    std::vector<double> hori(len), vert(len);
    qbo_boys_sequence(xsum * r2, angSum, hori.data());
    vert = hori;
    int nUpper = angSum;
    for (int k = 0; k < 3; ++k) {
        const int iSum = ang[k], iR = d.R.l[k];
        const double xML = d.cen[k] - d.L.c[k], xLR = drLR[k], xMC = drMC[k];
        const int nShift = nUpper - iSum;
        // vertSegHere = hori[end-iSum : end]
        double* here = hori.data() + (len - 1 - iSum);
        vertical_fill(here, iSum + 1, xML, xMC, xsum, 1.0);
        for (int sMin = 1; sMin <= nShift; ++sMin) {
            const int sMax = sMin + iSum;
            double* next = vert.data() + (len - 1 - sMax);
            vertical_push(next, here, iSum + 1, xML, xMC, xsum, 1.0);
            const double v = angular_shift(here, iSum + 1, iR, xLR);
            hori[len - 1 - sMin + 1] = v;
            here = hori.data() + (len - 1 - sMax);
            std::memcpy(here, next, sizeof(double) * (iSum + 1));
        }
        hori[len - 1 - nShift] = angular_shift(here, iSum + 1, iR, xLR);
        vert = hori;
        nUpper -= iSum;
    }
    return factor * hori[len - 1];
}

// modeTransfer (GaussianOrbitals.jl:529-538)
inline double mode_transfer(double p0m2, double p1m1, double p0m1, double m1m1, int i, int o,
                            const double xR12[2], const double xLR12[2], const double xS12[2]) {
    const double part1 = (i * m1m1 + (o - 1) * p0m2) / (2 * xS12[1]);
    const double part2 = ((xR12[0] * xLR12[0] + xR12[1] * xLR12[1]) * p0m1 + xS12[0] * p1m1) / xS12[1];
    return part1 - part2;
}

// angularCross! (GaussianOrbitals.jl:543-571); holder is (oSum+1) x angSpace, row-major here
void angular_cross(std::vector<double>& H, const double* data, int angSpace, int oSum,
                   const double xR12[2], const double xLR12[2], const double xS12[2]) {
    H.assign((oSum + 1) * angSpace, 0.0);
    auto at = [&](int r, int c) -> double& { return H[r * angSpace + c]; };
    for (int c = 0; c < angSpace; ++c) at(0, c) = data[c];
    for (int o = 1; o <= oSum; ++o) {
        const int n = angSpace - o - 1;
        double p1m1 = at(o - 1, n + 1);
        double p0m1 = at(o - 1, n);
        double m1m1 = n > 0 ? at(o - 1, n - 1) : 0.0;
        double p0m2 = o > 1 ? at(o - 2, n) : 0.0;
        for (int i = n; i >= 0; --i) {
            const double v = mode_transfer(p0m2, p1m1, p0m1, m1m1, i, o, xR12, xLR12, xS12);
            at(o, i) = v;
            p1m1 = p0m1;
            p0m1 = m1m1;
            m1m1 = i > 1 ? at(o - 1, i - 2) : 0.0;
            p0m2 = (i > 0 && o > 1) ? at(o - 2, i - 1) : 0.0;
        }
    }
}

// orbitalShift! (GaussianOrbitals.jl:581-592); data has length angSpace
double orbital_shift(double* data, int angSpace, int oSum, int iR, int oR, const double xR12[2],
                     const double xLR12[2], const double xS12[2]) {
    std::vector<double> H;
    angular_cross(H, data, angSpace, oSum, xR12, xLR12, xS12);
    const int ncol = angSpace - oSum;
    std::vector<double> slot(oSum + 1);
    for (int n = 0; n < ncol; ++n) {
        for (int r = 0; r <= oSum; ++r) slot[r] = H[r * angSpace + n];
        data[n] = angular_shift(slot.data(), oSum + 1, oR, xLR12[1]);
    }
    return angular_shift(data, ncol, iR, xLR12[0]);
}

// computePGTOrbTwoBodyRepulsion! (GaussianOrbitals.jl:594-663)
double prim_eri(const Product& d1, const Product& d2) {
    double drLR1[3], drLR2[3], drM12[3];
    int ijk[3], opq[3], ang[3], angSum = 0;
    for (int k = 0; k < 3; ++k) {
        drLR1[k] = d1.L.c[k] - d1.R.c[k];
        drLR2[k] = d2.L.c[k] - d2.R.c[k];
        drM12[k] = d1.cen[k] - d2.cen[k];
        ijk[k] = d1.L.l[k] + d1.R.l[k];
        opq[k] = d2.L.l[k] + d2.R.l[k];
        ang[k] = ijk[k] + opq[k];
        angSum += ang[k];
    }
    const double xR12[2] = {d1.R.a, d2.R.a};
    const double xS12[2] = {d1.xpn, d2.xpn};
    const double xpos1 = d1.L.a * d1.R.a / d1.xpn, xpos2 = d2.L.a * d2.R.a / d2.xpn;
    const double xsumpos = (xS12[0] * xS12[1]) / (xS12[0] + xS12[1]);
    const double xfactor = xsumpos / xS12[0];
    double m1 = 1.0, m2 = 1.0;
    for (int k = 0; k < 3; ++k) m1 *= std::exp(-xpos1 * drLR1[k] * drLR1[k]);
    for (int k = 0; k < 3; ++k) m2 *= std::exp(-xpos2 * drLR2[k] * drLR2[k]);
    const double pre1 = m1 / xS12[0], pre2 = m2 / xS12[1];
    const double factor = 2 * std::pow(kPi, 2.5) * pre1 * pre2 / std::sqrt(xS12[0] + xS12[1]);
    const double r2 = (drM12[0] * drM12[0] + drM12[1] * drM12[1]) + drM12[2] * drM12[2];
    const int len = angSum + 1;
    std::vector<double> hori(len), vert(len), tmp;
    qbo_boys_sequence(xsumpos * r2, angSum, hori.data());
    vert = hori;
    int nUpper = angSum;
    for (int k = 0; k < 3; ++k) {
        const int ioSum = ang[k], oSum = opq[k], iR = d1.R.l[k], oR = d2.R.l[k];
        const double xML1 = d1.cen[k] - d1.L.c[k];
        const double xLR12[2] = {drLR1[k], drLR2[k]};
        const double xM12 = drM12[k];
        const int nShift = nUpper - ioSum;
        double* here = hori.data() + (len - 1 - ioSum);
        vertical_fill(here, ioSum + 1, xML1, xM12, xS12[0], xfactor);
        for (int sMin = 1; sMin <= nShift; ++sMin) {
            const int sMax = sMin + ioSum;
            double* next = vert.data() + (len - 1 - sMax);
            vertical_push(next, here, ioSum + 1, xML1, xM12, xS12[0], xfactor);
            const double v = orbital_shift(here, ioSum + 1, oSum, iR, oR, xR12, xLR12, xS12);
            hori[len - 1 - sMin + 1] = v;
            here = hori.data() + (len - 1 - sMax);
            std::memcpy(here, next, sizeof(double) * (ioSum + 1));
        }
        hori[len - 1 - nShift] = orbital_shift(here, ioSum + 1, oSum, iR, oR, xR12, xLR12, xS12);
        vert = hori;
        nUpper -= ioSum;
    }
    return factor * hori[len - 1];
}

Prim make_prim(const double* c, double a, const int* l) {
    Prim p;
    for (int k = 0; k < 3; ++k) { p.c[k] = c[k]; p.l[k] = l[k]; }
    p.a = a;
    return p;
}

// Flattened basis: function f owns primitives [fp[f], fp[f+1]); each primitive
// has its own centre, Cartesian exponents, exponent and effective weight (the
// contraction coefficient with every normalisation factor already applied, as
// produced by buildOrbCoreWeight!, Framework.jl:748-773).
struct Basis {
    int nfun;
    const int* fp;
    const double* cen;
    const int* ijk;
    const double* alpha;
    const double* w;
    Prim prim(int p) const { return make_prim(cen + 3 * p, alpha[p], ijk + 3 * p); }
};

// getOrbLayoutIntegralCore! one-body (Framework.jl:505-523); kind 0=S 1=T 2=V
double contracted_1e(const Basis& b, int i, int j, int kind, int nnuc, const double* Z,
                     const double* R) {
    double res = 0.0;
    for (int pr = b.fp[j]; pr < b.fp[j + 1]; ++pr) {
        for (int pl = b.fp[i]; pl < b.fp[i + 1]; ++pl) {
            const Product d = make_product(b.prim(pl), b.prim(pr));
            double v;
            if (kind == 0) v = prim_overlap(d);
            else if (kind == 1) v = prim_kinetic(d);
            else {
                // CoulombMultiPointSampler: Σ_C Z_C (a|1/r_C|b), times testCharge −1
                // (GaussianOrbitals.jl:697-708; Samplers.jl:58)
                v = 0.0;
                for (int c = 0; c < nnuc; ++c) v += Z[c] * prim_nuclear(d, R + 3 * c);
                v *= -1.0;
            }
            res += v * (b.w[pl] * b.w[pr]);
        }
    }
    return res;
}

// getOrbLayoutIntegralCore! two-body (Framework.jl:526-554): Σ w·w·w·w (ab|cd)
double contracted_eri(const Basis& b, int i, int j, int k, int l) {
    double res = 0.0;
    for (int r2 = b.fp[l]; r2 < b.fp[l + 1]; ++r2)
        for (int l2 = b.fp[k]; l2 < b.fp[k + 1]; ++l2) {
            const double w2 = b.w[l2] * b.w[r2];
            const Product d2 = make_product(b.prim(l2), b.prim(r2));
            for (int r1 = b.fp[j]; r1 < b.fp[j + 1]; ++r1)
                for (int l1 = b.fp[i]; l1 < b.fp[i + 1]; ++l1) {
                    const Product d1 = make_product(b.prim(l1), b.prim(r1));
                    res += prim_eri(d1, d2) * (b.w[l1] * b.w[r1] * w2);
                }
        }
    return res;
}

void tri2d(int64_t n, int64_t& i, int64_t& j) {   // convertIndex1DtoTri2D (Iteration.jl:7-12), 1-based
    j = ((int64_t)std::floor(std::sqrt(8.0 * n - 6.9) - 1.0) >> 1) + 1;
    i = n - j * (j - 1) / 2;
}

}  // namespace

extern "C" {

double qbo_prim_overlap(const double* A, double a, const int* la, const double* B, double b,
                        const int* lb) {
    return prim_overlap(make_product(make_prim(A, a, la), make_prim(B, b, lb)));
}

double qbo_prim_kinetic(const double* A, double a, const int* la, const double* B, double b,
                        const int* lb) {
    return prim_kinetic(make_product(make_prim(A, a, la), make_prim(B, b, lb)));
}

double qbo_prim_nuclear(const double* A, double a, const int* la, const double* B, double b,
                        const int* lb, const double* C) {
    return prim_nuclear(make_product(make_prim(A, a, la), make_prim(B, b, lb)), C);
}

double qbo_prim_eri(const double* A, double a, const int* la, const double* B, double b,
                    const int* lb, const double* C, double c, const int* lc, const double* D,
                    double d, const int* ld) {
    return prim_eri(make_product(make_prim(A, a, la), make_prim(B, b, lb)),
                    make_product(make_prim(C, c, lc), make_prim(D, d, ld)));
}

// getOrbVectorIntegralCore! one-body, symmetric fill (Framework.jl:581-607).
// kind: 0 overlap, 1 kinetic, 2 nuclear attraction.  out is nfun x nfun column-major.
void qbo_one_body(int kind, int nfun, const int* fp, const double* cen, const int* ijk,
                  const double* alpha, const double* w, int nnuc, const double* Z,
                  const double* R, double* out) {
    const Basis b{nfun, fp, cen, ijk, alpha, w};
    const int64_t ntri = int64_t(nfun) * (nfun + 1) / 2;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t n = 1; n <= ntri; ++n) {
        int64_t i, j;
        tri2d(n, i, j);
        const double v = contracted_1e(b, int(i - 1), int(j - 1), kind, nnuc, Z, R);
        out[(i - 1) + (j - 1) * nfun] = v;
        out[(j - 1) + (i - 1) * nfun] = v;
    }
}

// getOrbVectorIntegralCore! two-body with the 8-fold scatter (Framework.jl:640-666).
// eri is nfun^4, column-major [i,j,k,l] in chemists' notation (ij|kl).
void qbo_eri_tensor(int nfun, const int* fp, const double* cen, const int* ijk,
                    const double* alpha, const double* w, double* eri) {
    const Basis b{nfun, fp, cen, ijk, alpha, w};
    const int64_t N = nfun;
    auto idx = [N](int64_t i, int64_t j, int64_t k, int64_t l) {
        return ((i - 1) + N * ((j - 1) + N * ((k - 1) + N * (l - 1))));
    };
    const int64_t m = N * (N + 1) / 2, total = m * (m + 1) / 2;
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t n = 1; n <= total; ++n) {
        int64_t p, q, i, j, k, l;
        tri2d(n, p, q);
        tri2d(p, i, j);
        tri2d(q, k, l);
        const double v = contracted_eri(b, int(i - 1), int(j - 1), int(k - 1), int(l - 1));
        eri[idx(i, j, k, l)] = v; eri[idx(j, i, k, l)] = v; eri[idx(i, j, l, k)] = v;
        eri[idx(j, i, l, k)] = v; eri[idx(k, l, i, j)] = v; eri[idx(k, l, j, i)] = v;
        eri[idx(l, k, i, j)] = v; eri[idx(l, k, j, i)] = v;
    }
}

// Contracted ERIs of an explicit list of function quartets (ij|kl), 0-based.
void qbo_eri_list(int nfun, const int* fp, const double* cen, const int* ijk,
                  const double* alpha, const double* w, int64_t nq, const int* quartets,
                  double* out) {
    const Basis b{nfun, fp, cen, ijk, alpha, w};
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t q = 0; q < nq; ++q) {
        const int* t = quartets + 4 * q;
        out[q] = contracted_eri(b, t[0], t[1], t[2], t[3]);
    }
}

// Direct J/K over a list of function quartets with degeneracy weights (the
// Fock contraction of getGcore, HartreeFock.jl:305-319, written for a quartet
// list instead of the stored tensor).  For each listed quartet with value v
// and weight g:  Jp[ij] += g D[kl] v, Jp[kl] += g D[ij] v,
//                Kp[ik] += g D[jl] v, Kp[jl] += g D[ik] v, Kp[il] += g D[jk] v,
//                Kp[jk] += g D[il] v.
// With the canonical list (i>=j, k>=l, ij>=kl) and g = (i!=j?2:1)(k!=l?2:1)(ij!=kl?2:1),
// J = (Jp + Jp^T)/4 and K = (Kp + Kp^T)/8.  Jp, Kp are accumulated (nfun^2, col-major).
void qbo_jk_list(int nfun, const int* fp, const double* cen, const int* ijk,
                 const double* alpha, const double* w, int64_t nq, const int* quartets,
                 const double* g, const double* D, double* Jp, double* Kp, int nthreads) {
    const Basis b{nfun, fp, cen, ijk, alpha, w};
    const int64_t N = nfun;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        std::vector<double> jl(N * N, 0.0), kl(N * N, 0.0);
#pragma omp for schedule(dynamic, 4)
        for (int64_t q = 0; q < nq; ++q) {
            const int* t = quartets + 4 * q;
            const int64_t i = t[0], j = t[1], k = t[2], l = t[3];
            const double v = contracted_eri(b, t[0], t[1], t[2], t[3]) * g[q];
            jl[i + N * j] += D[k + N * l] * v;
            jl[k + N * l] += D[i + N * j] * v;
            kl[i + N * k] += D[j + N * l] * v;
            kl[j + N * l] += D[i + N * k] * v;
            kl[i + N * l] += D[j + N * k] * v;
            kl[j + N * k] += D[i + N * l] * v;
        }
#pragma omp critical
        {
            for (int64_t x = 0; x < N * N; ++x) { Jp[x] += jl[x]; Kp[x] += kl[x]; }
        }
    }
}

int qbo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
