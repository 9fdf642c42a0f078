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
//
// Every routine is a template on the real type R.  R = double restates the
// reference as it runs (Float64); R = _Float128 (glibc's quad-precision math)
// evaluates the same definitions with 113-bit mantissas and serves as the
// exact value against which both the reference restatement and the GPU kernels
// are measured: the reference's electron-transfer step amplifies round-off by
// up to ~1e9 when the bra exponents are much larger than the ket exponents, so
// its Float64 results are not exact to 1e-12 in those cases.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {
_Float128 expf128(_Float128);
_Float128 logf128(_Float128);
_Float128 log10f128(_Float128);
_Float128 sqrtf128(_Float128);
_Float128 powf128(_Float128, _Float128);
_Float128 erff128(_Float128);
_Float128 tgammaf128(_Float128);
_Float128 lgammaf128(_Float128);
_Float128 fabsf128(_Float128);
_Float128 ceilf128(_Float128);
_Float128 floorf128(_Float128);
_Float128 roundf128(_Float128);
_Float128 acosf128(_Float128);
}

namespace {

typedef _Float128 quad;

inline double m_exp(double x) { return std::exp(x); }
inline quad m_exp(quad x) { return expf128(x); }
inline double m_log(double x) { return std::log(x); }
inline quad m_log(quad x) { return logf128(x); }
inline double m_log10(double x) { return std::log10(x); }
inline quad m_log10(quad x) { return log10f128(x); }
inline double m_sqrt(double x) { return std::sqrt(x); }
inline quad m_sqrt(quad x) { return sqrtf128(x); }
inline double m_pow(double x, double y) { return std::pow(x, y); }
inline quad m_pow(quad x, quad y) { return powf128(x, y); }
inline double m_erf(double x) { return std::erf(x); }
inline quad m_erf(quad x) { return erff128(x); }
inline double m_tgamma(double x) { return std::tgamma(x); }
inline quad m_tgamma(quad x) { return tgammaf128(x); }
inline double m_lgamma(double x) { return std::lgamma(x); }
inline quad m_lgamma(quad x) { return lgammaf128(x); }
inline double m_fabs(double x) { return std::fabs(x); }
inline quad m_fabs(quad x) { return fabsf128(x); }
inline double m_ceil(double x) { return std::ceil(x); }
inline quad m_ceil(quad x) { return ceilf128(x); }
inline double m_round(double x) { return std::round(x); }
inline quad m_round(quad x) { return roundf128(x); }
inline bool m_isinf(double x) { return std::isinf(x); }
inline bool m_isinf(quad x) { return x > (quad)1e4000L || x < -(quad)1e4000L; }

template <class R> struct Tr;
template <> struct Tr<double> {
    // PowersOfPi (src/Lexicons.jl:1-8): correctly rounded pi^0.5, pi, pi^2.5
    static double pi() { return 3.14159265358979323846264338327950288; }
    static double sqrtpi() { return 1.77245385090551602729816748334114518; }
    static double pi25() { return 17.4934183276248628462628216798715; }
    static constexpr double eps = 2.220446049250313e-16;
    static constexpr double atol = 4e-16;   // getAtolVal(Float64) (src/Arithmetic.jl:42)
    static constexpr int digits = 15;       // getAtolDigits(Float64) (src/Arithmetic.jl:8-16)
};
template <> struct Tr<quad> {
    static quad pi() { return acosf128((quad)-1); }
    static quad sqrtpi() { return sqrtf128(pi()); }
    static quad pi25() { return pi() * pi() * sqrtpi(); }
    static constexpr double eps = 1.925929944387236e-34;
    static constexpr double atol = 3e-34;   // ceil(3eps/2, sigdigits=1) for 113-bit mantissas
    static constexpr int digits = 33;
};

// ---------------------------------------------------------------------------
// Regularised lower incomplete gamma P(a, x), a > 0, x >= 0.
template <class R>
R gamma_p(R a, R x) {
    if (x <= 0) return 0;
    const R gln = m_lgamma(a);
    const R tiny = (R)Tr<R>::eps * (R)0.05;
    if (x < a + 1) {                         // series (Numerical Recipes gser)
        R ap = a, sum = 1 / a, del = sum;
        for (int n = 0; n < 100000; ++n) {
            ap += 1;
            del *= x / ap;
            sum += del;
            if (m_fabs(del) < m_fabs(sum) * tiny) break;
        }
        return sum * m_exp(-x + a * m_log(x) - gln);
    }
    // continued fraction for Q (Numerical Recipes gcf, modified Lentz)
    const R fpmin = (R)1e-300;
    R b = x + 1 - a, c = 1 / fpmin, d = 1 / b, h = d;
    for (int i = 1; i < 100000; ++i) {
        const R an = -i * (i - a);
        b += 2;
        d = an * d + b;
        if (m_fabs(d) < fpmin) d = fpmin;
        c = b + an / c;
        if (m_fabs(c) < fpmin) c = fpmin;
        d = 1 / d;
        const R del = d * c;
        h *= del;
        if (m_fabs(del - 1) < tiny) break;
    }
    return 1 - m_exp(-x + a * m_log(x) - gln) * h;
}

// directComputeBoysFunc (BoysFunction.jl:7-24)
template <class R>
R direct_boys(R x, int n) {
    const R z = (R)n + (R)0.5;
    const R p = gamma_p(z, x);
    if (p == 0) return 0;
    R res;
    if (z < 23) {
        const R part1 = m_tgamma(z) * p;
        const R part2 = m_pow(x, z);
        res = m_isinf(part2) ? m_exp(m_log(part1) - z * m_log(x)) : part1 / part2;
    } else {
        res = m_exp(m_lgamma(z) + m_log(p) - z * m_log(x));
    }
    return res / 2;
}

// initializeUpperOrder (BoysFunction.jl:27-31)
// At x = n = 1 the ratio is 1 and the formula diverges (the reference's Int(ceil(Inf))
// raises InexactError there); its limit is taken, so that min(., 6n) picks 6n.
template <class R>
int upper_order(R x, int n) {
    const R ratio = ((R)n == x) ? (R)n : (R)n / x;
    const R lg = m_fabs(m_log10(ratio));
    if (!(lg > 0)) return 1 << 30;
    const R up = m_ceil((R)Tr<R>::digits / lg + n);
    if (up > (R)(1 << 30)) return 1 << 30;
    const int res = int(up);
    return res + (res & 1);
}

// recursiveGetBoysFuncDn (BoysFunction.jl:33-40)
template <class R>
R boys_down(R x, int m, R val, int n) {
    const R ex = m_exp(-x);
    for (int i = m - 1; i >= n; --i) val = (2 * x * val + ex) / (2 * i + 1);
    return val;
}

// computeBoysFunc (BoysFunction.jl:52-64)
template <class R>
R boys(R x, int n) {
    if (n == 0) {
        if (x < (R)Tr<R>::atol) return 1;
        const R r = m_sqrt(x);
        return Tr<R>::sqrtpi() * m_erf(r) / (2 * r);
    }
    if (x < (R)Tr<R>::atol) return (R)1 / (2 * n + 1);
    const int nup = std::min(upper_order(x, n), 6 * n);
    const R fup = direct_boys(x, nup);
    return boys_down(x, nup, fup, n);
}

// computeBoysSequence (BoysFunction.jl:67-77): out[0..n]
template <class R>
void boys_sequence(R x, int n, R* out) {
    out[0] = boys(x, 0);
    if (n > 0) out[n] = boys(x, n);
    for (int m = n; m >= 2; --m) out[m - 1] = boys_down(x, m, out[m], m - 1);
}

}  // namespace

extern "C" {

double qbo_boys(double x, int n) { return boys<double>(x, n); }

void qbo_boys_sequence(double x, int n, double* out) { boys_sequence<double>(x, n, out); }

double qbo_boys_q(double x, int n) { return (double)boys<quad>((quad)x, n); }

}  // extern "C"

namespace {

double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    double r = 1.0;
    for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
    return std::round(r);
}

template <class R>
R ipow(R x, int e) {
    R r = 1;
    for (int i = 0; i < e; ++i) r *= x;
    return r;
}

// computePGTOrbOverlapAxialFactor + oddFactorial (GaussianOrbitals.jl:94-97, Arithmetic.jl:101-107)
template <class R>
R axial_factor(R xsum, int degree) {
    R f = 1;
    if (degree > 0) {
        const R coeff = 1 / (2 * xsum);
        for (int i = 1; i <= 2 * degree - 1; i += 2) f *= i * coeff;
    }
    return Tr<R>::sqrtpi() / m_sqrt(xsum) * f;
}

// computeGaussProd (Arithmetic.jl:110-120)
template <class R>
R gauss_prod(R dxML, R dxMR, int lL, int lR, int lx) {
    const int lb = std::max(-lx, lx - 2 * lR), ub = std::min(lx, 2 * lL - lx);
    R res = 0;
    for (int q = lb; q <= ub; q += 2) {
        const int i = (lx + q) >> 1, j = (lx - q) >> 1;
        res += (R)binom(lL, i) * (R)binom(lR, j) * ipow(dxML, lL - i) * ipow(dxMR, lR - j);
    }
    return res;
}

// computeAxialPGTOrbOverlap, adaptive form (GaussianOrbitals.jl:110-138)
template <class R>
R axial_overlap(R xsum, R xpos, R xML, R xMR, int iL, int iR) {
    const R dx = xMR - xML;
    if (iL == 0 && iR == 0) return axial_factor(xsum, 0) * m_exp(-xpos * dx * dx);
    if (dx == 0) {   // concentric: computeGaussProd(iL,iR,2j) selects 2j == iL+iR
        return ((iL + iR) % 2 == 0) ? axial_factor(xsum, (iL + iR) / 2) : (R)0;
    }
    R res = 0;
    for (int j = 0; j <= (iL + iR) / 2; ++j)
        res += gauss_prod(xML, xMR, iL, iR, 2 * j) * axial_factor(xsum, j);
    return res * m_exp(-xpos * dx * dx);
}

template <class R>
struct Prim {
    R c[3];
    R a;
    int l[3];
};

template <class R>
bool same_prim(const Prim<R>& x, const Prim<R>& y) {
    return x.a == y.a && x.c[0] == y.c[0] && x.c[1] == y.c[1] && x.c[2] == y.c[2] &&
           x.l[0] == y.l[0] && x.l[1] == y.l[1] && x.l[2] == y.l[2];
}

// GaussProductInfo (GaussianOrbitals.jl:18-37)
template <class R>
struct Product {
    Prim<R> L, Rt;
    R cen[3];
    R xpn;
    bool sym;
};

template <class R>
Product<R> make_product(const Prim<R>& L, const Prim<R>& Rt) {
    Product<R> p{L, Rt, {0, 0, 0}, L.a + Rt.a, same_prim(L, Rt)};
    for (int k = 0; k < 3; ++k)
        p.cen[k] = p.sym ? L.c[k] : (L.a * L.c[k] + Rt.a * Rt.c[k]) / p.xpn;
    return p;
}

// computePGTOrbOverlap / computePGTOrbOverlap! (GaussianOrbitals.jl:147-179)
template <class R>
R prim_overlap(const Product<R>& d) {
    if (d.sym) {
        R r = 1;
        for (int k = 0; k < 3; ++k) r *= axial_factor(2 * d.L.a, d.L.l[k]);
        return r;
    }
    const R xpos = d.L.a * d.Rt.a / d.xpn;
    R r = 1;
    for (int k = 0; k < 3; ++k)
        r *= axial_overlap(d.xpn, xpos, d.cen[k] - d.L.c[k], d.cen[k] - d.Rt.c[k], d.L.l[k], d.Rt.l[k]);
    return r;
}

// computePGTOrbMultipoleMoment (GaussianOrbitals.jl:184-202): a primitive with itself,
// monomial prod_k (x_k - C_k)^n_k
template <class R>
R prim_multipole_sym(const Prim<R>& p, const R C[3], const int n[3]) {
    R res = 1;
    for (int k = 0; k < 3; ++k) {
        const R dx = p.c[k] - C[k];
        const int m = (dx == 0) ? 0 : n[k];
        R temp = 0;
        for (int q = 0; q <= m; ++q) {
            const int l = n[k] - q;
            if (l % 2 == 0) temp += (R)binom(n[k], q) * ipow(dx, q) * axial_factor(2 * p.a, p.l[k] + (l >> 1));
        }
        res *= temp;
    }
    return res;
}

// computePGTOrbMultipoleMoment! (GaussianOrbitals.jl:204-247): binomial expansion of
// (x - C)^n about the right centre (or the left one when C sits on it)
template <class R>
R prim_multipole(const Product<R>& d, const R C[3], const int n[3]) {
    if (n[0] + n[1] + n[2] == 0) return prim_overlap(d);
    if (d.sym) return prim_multipole_sym(d.L, C, n);
    const R xpos = d.L.a * d.Rt.a / d.xpn;
    R res = 1;
    for (int k = 0; k < 3; ++k) {
        R xL = d.L.c[k], xR = d.Rt.c[k];
        int iL = d.L.l[k], iR = d.Rt.l[k];
        const R dx = xR - C[k];
        int m = n[k];
        if (dx == 0) {
            m = 0;
        } else if (xL == C[k]) {
            std::swap(xL, xR);
            std::swap(iL, iR);
            m = 0;
        }
        R temp = 0;
        for (int q = 0; q <= m; ++q)
            temp += (R)binom(n[k], q) * ipow(dx, q) *
                    axial_overlap(d.xpn, xpos, d.cen[k] - xL, d.cen[k] - xR, iL, iR + n[k] - q);
        res *= temp;
    }
    return res;
}

// computeAxialPGTOrbCoordDiff! (GaussianOrbitals.jl:258-281)
template <class R>
R axial_diff(int degree, R xL, R xR, R xML, R xMR, int iL, int iR) {
    if (degree < 1) {
        const R xsum = xL + xR;
        return axial_overlap(xsum, xL * xR / xsum, xML, xMR, iL, iR);
    }
    const R dn = iR < 1 ? (R)0 : axial_diff(degree - 1, xL, xR, xML, xMR, iL, iR - 1);
    const R up = axial_diff(degree - 1, xL, xR, xML, xMR, iL, iR + 1);
    return dn * iR - up * 2 * xR;
}

// computeAxialPGTOrbCoordDiff, concentric equal-exponent form (GaussianOrbitals.jl:283-292)
template <class R>
R axial_diff_sym(int degree, R xpn, int iL, int iR) {
    if (degree < 1) {
        return ((iL + iR) % 2 == 0) ? axial_factor(2 * xpn, (iL + iR) / 2) : (R)0;
    }
    const R dn = iR < 1 ? (R)0 : axial_diff_sym(degree - 1, xpn, iL, iR - 1);
    const R up = axial_diff_sym(degree - 1, xpn, iL, iR + 1);
    return dn * iR - up * 2 * xpn;
}

// kinetic = Σ_axes (−½)·∂²-sandwich (Samplers.jl:81-107; GaussianOrbitals.jl:295-363,686-694)
template <class R>
R prim_kinetic(const Product<R>& d) {
    R res[3] = {1, 1, 1};
    for (int k = 0; k < 3; ++k) {
        R diff, ovl;
        if (d.sym) {
            diff = axial_diff_sym(2, d.L.a, d.L.l[k], d.L.l[k]);
            ovl = axial_factor(2 * d.L.a, d.L.l[k]);
        } else {
            const R xML = d.cen[k] - d.L.c[k], xMR = d.cen[k] - d.Rt.c[k];
            diff = axial_diff(2, d.L.a, d.Rt.a, xML, xMR, d.L.l[k], d.Rt.l[k]);
            ovl = axial_overlap(d.xpn, d.L.a * d.Rt.a / d.xpn, xML, xMR, d.L.l[k], d.Rt.l[k]);
        }
        res[k] *= diff;
        for (int o = 0; o < 3; ++o)
            if (o != k) res[o] *= ovl;
    }
    const R h = (R)-0.5;
    return (h * res[0] + h * res[1]) + h * res[2];
}

// --- Obara–Saika Coulomb recursions (GaussianOrbitals.jl:378-663) -----------
// Buffers are 0-based; "end-k" of the reference is index (len-1-k).

// vertTransfer (GaussianOrbitals.jl:386-391)
template <class R>
inline R vert_transfer(R p0m1, R p1m1, R p0m2, R p1m2, int iL, R xML, R xMC, R xsum, R factor) {
    const R part1 = xML * p0m1 - factor * xMC * p1m1;
    const R part2 = (iL - 1) * (p0m2 - factor * p1m2) * (1 / (2 * xsum));
    return part1 + part2;
}

// verticalFill! (GaussianOrbitals.jl:401-418); h has length iSum+1
template <class R>
void vertical_fill(R* h, int len, R xML, R xMC, R xsum, R factor) {
    const int iSum = len - 1;
    for (int n = 1; n <= iSum; ++n) {
        R b0 = h[len - 1 - n], b1 = h[len - 1 - n + 1], b2 = 0, b3 = 0;
        for (int iMax = 1; iMax <= n; ++iMax) {
            const R p0 = b0, p1 = b1;
            const R here = vert_transfer(b0, b1, b2, b3, iMax, xML, xMC, xsum, factor);
            if (iMax < n) { b0 = here; b1 = h[len - 1 - n + iMax + 1]; b2 = p0; b3 = p1; }
            h[len - 1 - n + iMax] = here;
        }
    }
}

// verticalPush! (GaussianOrbitals.jl:423-439)
template <class R>
void vertical_push(R* h, const R* data, int len, R xML, R xMC, R xsum, R factor) {
    const int iSum = len - 1;
    R b0 = h[0], b1 = data[0], b2 = 0, b3 = 0;
    for (int i = 1; i <= iSum; ++i) {
        const R here = vert_transfer(b0, b1, b2, b3, i, xML, xMC, xsum, factor);
        h[i] = here;
        if (i < iSum) { const R a = b0, b = b1; b0 = here; b1 = data[i]; b2 = a; b3 = b; }
    }
}

// angularShift! (GaussianOrbitals.jl:446-454); operates on the last iR+1 entries of h[0..len)
template <class R>
R angular_shift(R* h, int len, int iR, R xLR) {
    R* seg = h + (len - 1 - iR);
    for (int y = 1; y <= iR; ++y)
        for (int x = 1; x <= iR + 1 - y; ++x) seg[x - 1] = seg[x] + xLR * seg[x - 1];
    return seg[0];
}

// computePGTOrbOneBodyRepulsion! (GaussianOrbitals.jl:478-522)
template <class R>
R prim_nuclear(const Product<R>& d, const R C[3]) {
    R drLR[3], drMC[3];
    int ang[3], angSum = 0;
    for (int k = 0; k < 3; ++k) {
        drLR[k] = d.L.c[k] - d.Rt.c[k];
        drMC[k] = d.cen[k] - C[k];
        ang[k] = d.L.l[k] + d.Rt.l[k];
        angSum += ang[k];
    }
    const R xsum = d.xpn, xpos = d.L.a * d.Rt.a / xsum;
    R mixed = 1;
    for (int k = 0; k < 3; ++k) mixed *= m_exp(-xpos * drLR[k] * drLR[k]);
    const R factor = 2 * Tr<R>::pi() * (mixed / xsum);
    const R r2 = (drMC[0] * drMC[0] + drMC[1] * drMC[1]) + drMC[2] * drMC[2];
    const int len = angSum + 1;
    std::vector<R> hori(len), vert(len);
    boys_sequence<R>(xsum * r2, angSum, hori.data());
    vert = hori;
    int nUpper = angSum;
    for (int k = 0; k < 3; ++k) {
        const int iSum = ang[k], iR = d.Rt.l[k];
        const R xML = d.cen[k] - d.L.c[k], xLR = drLR[k], xMC = drMC[k];
        const int nShift = nUpper - iSum;
        R* here = hori.data() + (len - 1 - iSum);
        vertical_fill(here, iSum + 1, xML, xMC, xsum, (R)1);
        for (int sMin = 1; sMin <= nShift; ++sMin) {
            const int sMax = sMin + iSum;
            R* next = vert.data() + (len - 1 - sMax);
            vertical_push(next, here, iSum + 1, xML, xMC, xsum, (R)1);
            const R v = angular_shift(here, iSum + 1, iR, xLR);
            hori[len - 1 - sMin + 1] = v;
            here = hori.data() + (len - 1 - sMax);
            std::memcpy((void*)here, (const void*)next, sizeof(R) * (iSum + 1));
        }
        hori[len - 1 - nShift] = angular_shift(here, iSum + 1, iR, xLR);
        vert = hori;
        nUpper -= iSum;
    }
    return factor * hori[len - 1];
}

// modeTransfer (GaussianOrbitals.jl:529-538)
template <class R>
inline R mode_transfer(R p0m2, R p1m1, R p0m1, R m1m1, int i, int o, const R xR12[2], const R xLR12[2],
                       const R xS12[2]) {
    const R part1 = (i * m1m1 + (o - 1) * p0m2) / (2 * xS12[1]);
    const R part2 = ((xR12[0] * xLR12[0] + xR12[1] * xLR12[1]) * p0m1 + xS12[0] * p1m1) / xS12[1];
    return part1 - part2;
}

// angularCross! (GaussianOrbitals.jl:543-571); holder is (oSum+1) x angSpace, row-major here
template <class R>
void angular_cross(std::vector<R>& H, const R* data, int angSpace, int oSum, const R xR12[2], const R xLR12[2],
                   const R xS12[2]) {
    H.assign((oSum + 1) * angSpace, (R)0);
    auto at = [&](int r, int c) -> R& { return H[r * angSpace + c]; };
    for (int c = 0; c < angSpace; ++c) at(0, c) = data[c];
    for (int o = 1; o <= oSum; ++o) {
        const int n = angSpace - o - 1;
        R p1m1 = at(o - 1, n + 1);
        R p0m1 = at(o - 1, n);
        R m1m1 = n > 0 ? at(o - 1, n - 1) : (R)0;
        R p0m2 = o > 1 ? at(o - 2, n) : (R)0;
        for (int i = n; i >= 0; --i) {
            const R v = mode_transfer(p0m2, p1m1, p0m1, m1m1, i, o, xR12, xLR12, xS12);
            at(o, i) = v;
            p1m1 = p0m1;
            p0m1 = m1m1;
            m1m1 = i > 1 ? at(o - 1, i - 2) : (R)0;
            p0m2 = (i > 0 && o > 1) ? at(o - 2, i - 1) : (R)0;
        }
    }
}

// orbitalShift! (GaussianOrbitals.jl:581-592); data has length angSpace
template <class R>
R orbital_shift(R* data, int angSpace, int oSum, int iR, int oR, const R xR12[2], const R xLR12[2],
                const R xS12[2]) {
    std::vector<R> H;
    angular_cross(H, data, angSpace, oSum, xR12, xLR12, xS12);
    const int ncol = angSpace - oSum;
    std::vector<R> slot(oSum + 1);
    for (int n = 0; n < ncol; ++n) {
        for (int r = 0; r <= oSum; ++r) slot[r] = H[r * angSpace + n];
        data[n] = angular_shift(slot.data(), oSum + 1, oR, xLR12[1]);
    }
    return angular_shift(data, ncol, iR, xLR12[0]);
}

// computePGTOrbTwoBodyRepulsion! (GaussianOrbitals.jl:594-663)
template <class R>
R prim_eri(const Product<R>& d1, const Product<R>& d2) {
    R drLR1[3], drLR2[3], drM12[3];
    int opq[3], ang[3], angSum = 0;
    for (int k = 0; k < 3; ++k) {
        drLR1[k] = d1.L.c[k] - d1.Rt.c[k];
        drLR2[k] = d2.L.c[k] - d2.Rt.c[k];
        drM12[k] = d1.cen[k] - d2.cen[k];
        opq[k] = d2.L.l[k] + d2.Rt.l[k];
        ang[k] = d1.L.l[k] + d1.Rt.l[k] + opq[k];
        angSum += ang[k];
    }
    const R xR12[2] = {d1.Rt.a, d2.Rt.a};
    const R xS12[2] = {d1.xpn, d2.xpn};
    const R xpos1 = d1.L.a * d1.Rt.a / d1.xpn, xpos2 = d2.L.a * d2.Rt.a / d2.xpn;
    const R xsumpos = (xS12[0] * xS12[1]) / (xS12[0] + xS12[1]);
    const R xfactor = xsumpos / xS12[0];
    R m1 = 1, m2 = 1;
    for (int k = 0; k < 3; ++k) m1 *= m_exp(-xpos1 * drLR1[k] * drLR1[k]);
    for (int k = 0; k < 3; ++k) m2 *= m_exp(-xpos2 * drLR2[k] * drLR2[k]);
    const R pre1 = m1 / xS12[0], pre2 = m2 / xS12[1];
    const R factor = 2 * Tr<R>::pi25() * pre1 * pre2 / m_sqrt(xS12[0] + xS12[1]);
    const R r2 = (drM12[0] * drM12[0] + drM12[1] * drM12[1]) + drM12[2] * drM12[2];
    const int len = angSum + 1;
    std::vector<R> hori(len), vert(len);
    boys_sequence<R>(xsumpos * r2, angSum, hori.data());
    vert = hori;
    int nUpper = angSum;
    for (int k = 0; k < 3; ++k) {
        const int ioSum = ang[k], oSum = opq[k], iR = d1.Rt.l[k], oR = d2.Rt.l[k];
        const R xML1 = d1.cen[k] - d1.L.c[k];
        const R xLR12[2] = {drLR1[k], drLR2[k]};
        const R xM12 = drM12[k];
        const int nShift = nUpper - ioSum;
        R* here = hori.data() + (len - 1 - ioSum);
        vertical_fill(here, ioSum + 1, xML1, xM12, xS12[0], xfactor);
        for (int sMin = 1; sMin <= nShift; ++sMin) {
            const int sMax = sMin + ioSum;
            R* next = vert.data() + (len - 1 - sMax);
            vertical_push(next, here, ioSum + 1, xML1, xM12, xS12[0], xfactor);
            const R v = orbital_shift(here, ioSum + 1, oSum, iR, oR, xR12, xLR12, xS12);
            hori[len - 1 - sMin + 1] = v;
            here = hori.data() + (len - 1 - sMax);
            std::memcpy((void*)here, (const void*)next, sizeof(R) * (ioSum + 1));
        }
        hori[len - 1 - nShift] = orbital_shift(here, ioSum + 1, oSum, iR, oR, xR12, xLR12, xS12);
        vert = hori;
        nUpper -= ioSum;
    }
    return factor * hori[len - 1];
}

template <class R>
Prim<R> make_prim(const double* c, double a, const int* l) {
    Prim<R> p;
    for (int k = 0; k < 3; ++k) { p.c[k] = (R)c[k]; p.l[k] = l[k]; }
    p.a = (R)a;
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
    template <class R>
    Prim<R> prim(int p) const { return make_prim<R>(cen + 3 * p, alpha[p], ijk + 3 * p); }
};

// getOrbLayoutIntegralCore! one-body (Framework.jl:505-523); kind 0=S 1=T 2=V
template <class R>
R contracted_1e(const Basis& b, int i, int j, int kind, int nnuc, const double* Z, const double* Rn) {
    R res = 0;
    for (int pr = b.fp[j]; pr < b.fp[j + 1]; ++pr) {
        for (int pl = b.fp[i]; pl < b.fp[i + 1]; ++pl) {
            const Product<R> d = make_product(b.prim<R>(pl), b.prim<R>(pr));
            R v;
            if (kind == 0) v = prim_overlap(d);
            else if (kind == 1) v = prim_kinetic(d);
            else {
                // CoulombMultiPointSampler: Σ_C Z_C (a|1/r_C|b), times testCharge −1
                // (GaussianOrbitals.jl:697-708; Samplers.jl:58)
                v = 0;
                for (int c = 0; c < nnuc; ++c) {
                    const R C3[3] = {(R)Rn[3 * c], (R)Rn[3 * c + 1], (R)Rn[3 * c + 2]};
                    v += (R)Z[c] * prim_nuclear(d, C3);
                }
                v *= -1;
            }
            res += v * ((R)b.w[pl] * (R)b.w[pr]);
        }
    }
    return res;
}

// getOrbLayoutIntegralCore! one-body with the multipole sampler (Framework.jl:505-523,
// Samplers.jl:19-21)
template <class R>
R contracted_multipole(const Basis& b, int i, int j, const R C[3], const int n[3]) {
    R res = 0;
    for (int pr = b.fp[j]; pr < b.fp[j + 1]; ++pr)
        for (int pl = b.fp[i]; pl < b.fp[i + 1]; ++pl) {
            const Product<R> d = make_product(b.prim<R>(pl), b.prim<R>(pr));
            res += prim_multipole(d, C, n) * ((R)b.w[pl] * (R)b.w[pr]);
        }
    return res;
}

// getOrbLayoutIntegralCore! two-body (Framework.jl:526-554): Σ w·w·w·w (ab|cd)
template <class R>
R contracted_eri(const Basis& b, int i, int j, int k, int l) {
    R res = 0;
    for (int r2 = b.fp[l]; r2 < b.fp[l + 1]; ++r2)
        for (int l2 = b.fp[k]; l2 < b.fp[k + 1]; ++l2) {
            const R w2 = (R)b.w[l2] * (R)b.w[r2];
            const Product<R> d2 = make_product(b.prim<R>(l2), b.prim<R>(r2));
            for (int r1 = b.fp[j]; r1 < b.fp[j + 1]; ++r1)
                for (int l1 = b.fp[i]; l1 < b.fp[i + 1]; ++l1) {
                    const Product<R> d1 = make_product(b.prim<R>(l1), b.prim<R>(r1));
                    res += prim_eri(d1, d2) * ((R)b.w[l1] * (R)b.w[r1] * w2);
                }
        }
    return res;
}

void tri2d(int64_t n, int64_t& i, int64_t& j) {   // convertIndex1DtoTri2D (Iteration.jl:7-12), 1-based
    j = ((int64_t)std::floor(std::sqrt(8.0 * n - 6.9) - 1.0) >> 1) + 1;
    i = n - j * (j - 1) / 2;
}

template <class R>
void one_body(int kind, const Basis& b, int nnuc, const double* Z, const double* Rn, double* out) {
    const int nfun = b.nfun;
    const int64_t ntri = int64_t(nfun) * (nfun + 1) / 2;
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t n = 1; n <= ntri; ++n) {
        int64_t i, j;
        tri2d(n, i, j);
        const double v = (double)contracted_1e<R>(b, int(i - 1), int(j - 1), kind, nnuc, Z, Rn);
        out[(i - 1) + (j - 1) * nfun] = v;
        out[(j - 1) + (i - 1) * nfun] = v;
    }
}

template <class R>
void eri_tensor(const Basis& b, double* eri) {
    const int64_t N = b.nfun;
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
        const double v = (double)contracted_eri<R>(b, int(i - 1), int(j - 1), int(k - 1), int(l - 1));
        eri[idx(i, j, k, l)] = v; eri[idx(j, i, k, l)] = v; eri[idx(i, j, l, k)] = v;
        eri[idx(j, i, l, k)] = v; eri[idx(k, l, i, j)] = v; eri[idx(k, l, j, i)] = v;
        eri[idx(l, k, i, j)] = v; eri[idx(l, k, j, i)] = v;
    }
}

template <class R>
void eri_list(const Basis& b, int64_t nq, const int* quartets, double* out) {
#pragma omp parallel for schedule(dynamic, 8)
    for (int64_t q = 0; q < nq; ++q) {
        const int* t = quartets + 4 * q;
        out[q] = (double)contracted_eri<R>(b, t[0], t[1], t[2], t[3]);
    }
}

template <class R>
void jk_list(const Basis& b, int64_t nq, const int* quartets, const double* g, const double* D, double* Jp,
             double* Kp) {
    const int64_t N = b.nfun;
#pragma omp parallel
    {
        std::vector<R> jl(N * N, (R)0), kl(N * N, (R)0);
#pragma omp for schedule(dynamic, 4)
        for (int64_t q = 0; q < nq; ++q) {
            const int* t = quartets + 4 * q;
            const int64_t i = t[0], j = t[1], k = t[2], l = t[3];
            const R v = contracted_eri<R>(b, t[0], t[1], t[2], t[3]) * (R)g[q];
            jl[i + N * j] += (R)D[k + N * l] * v;
            jl[k + N * l] += (R)D[i + N * j] * v;
            kl[i + N * k] += (R)D[j + N * l] * v;
            kl[j + N * l] += (R)D[i + N * k] * v;
            kl[i + N * l] += (R)D[j + N * k] * v;
            kl[j + N * k] += (R)D[i + N * l] * v;
        }
#pragma omp critical
        {
            for (int64_t x = 0; x < N * N; ++x) { Jp[x] += (double)jl[x]; Kp[x] += (double)kl[x]; }
        }
    }
}

template <class R>
Product<R> prod_of(const double* A, double a, const int* la, const double* B, double b, const int* lb) {
    return make_product(make_prim<R>(A, a, la), make_prim<R>(B, b, lb));
}

// multipoleMoments (Interface.jl:95): nfun x nfun, column-major, both triangles
// (getOrbVectorIntegralCore! one-body, Framework.jl:581-607).
template <class R>
void multipole_matrix(const Basis& b, const double* C, const int* n, double* out) {
    const R Cr[3] = {(R)C[0], (R)C[1], (R)C[2]};
    const int N = b.nfun;
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < N; ++j)
        for (int i = 0; i <= j; ++i) {
            const double v = (double)contracted_multipole<R>(b, i, j, Cr, n);
            out[i + (size_t)N * j] = v;
            out[j + (size_t)N * i] = v;
        }
}

}  // namespace

extern "C" {

double qbo_prim_overlap(const double* A, double a, const int* la, const double* B, double b, const int* lb) {
    return prim_overlap(prod_of<double>(A, a, la, B, b, lb));
}

double qbo_prim_kinetic(const double* A, double a, const int* la, const double* B, double b, const int* lb) {
    return prim_kinetic(prod_of<double>(A, a, la, B, b, lb));
}

double qbo_prim_nuclear(const double* A, double a, const int* la, const double* B, double b, const int* lb,
                        const double* C) {
    return prim_nuclear(prod_of<double>(A, a, la, B, b, lb), C);
}

double qbo_prim_eri(const double* A, double a, const int* la, const double* B, double b, const int* lb,
                    const double* C, double c, const int* lc, const double* D, double d, const int* ld) {
    return prim_eri(prod_of<double>(A, a, la, B, b, lb), prod_of<double>(C, c, lc, D, d, ld));
}

// getOrbVectorIntegralCore! one-body, symmetric fill (Framework.jl:581-607).
// kind: 0 overlap, 1 kinetic, 2 nuclear attraction.  out is nfun x nfun column-major.
// prec: 0 Float64 (the reference as it runs), 1 quad precision (exact values).
void qbo_one_body(int kind, int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                  const double* w, int nnuc, const double* Z, const double* R, double* out) {
    one_body<double>(kind, Basis{nfun, fp, cen, ijk, alpha, w}, nnuc, Z, R, out);
}
void qbo_one_body_q(int kind, int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                    const double* w, int nnuc, const double* Z, const double* R, double* out) {
    one_body<quad>(kind, Basis{nfun, fp, cen, ijk, alpha, w}, nnuc, Z, R, out);
}

void qbo_multipole(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                   const double* w, const double* C, const int* n, double* out) {
    multipole_matrix<double>(Basis{nfun, fp, cen, ijk, alpha, w}, C, n, out);
}
void qbo_multipole_q(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                     const double* w, const double* C, const int* n, double* out) {
    multipole_matrix<quad>(Basis{nfun, fp, cen, ijk, alpha, w}, C, n, out);
}

// getOrbVectorIntegralCore! two-body with the 8-fold scatter (Framework.jl:640-666).
// eri is nfun^4, column-major [i,j,k,l] in chemists' notation (ij|kl).
void qbo_eri_tensor(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                    const double* w, double* eri) {
    eri_tensor<double>(Basis{nfun, fp, cen, ijk, alpha, w}, eri);
}
void qbo_eri_tensor_q(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                      const double* w, double* eri) {
    eri_tensor<quad>(Basis{nfun, fp, cen, ijk, alpha, w}, eri);
}

// Contracted ERIs of an explicit list of function quartets (ij|kl), 0-based.
void qbo_eri_list(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                  const double* w, int64_t nq, const int* quartets, double* out) {
    eri_list<double>(Basis{nfun, fp, cen, ijk, alpha, w}, nq, quartets, out);
}
void qbo_eri_list_q(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                    const double* w, int64_t nq, const int* quartets, double* out) {
    eri_list<quad>(Basis{nfun, fp, cen, ijk, alpha, w}, nq, quartets, out);
}

// Direct J/K over a list of function quartets with degeneracy weights (the
// Fock contraction of getGcore, HartreeFock.jl:305-319, written for a quartet
// list instead of the stored tensor).  For each listed quartet with value v
// and weight g:  Jp[ij] += g D[kl] v, Jp[kl] += g D[ij] v,
//                Kp[ik] += g D[jl] v, Kp[jl] += g D[ik] v, Kp[il] += g D[jk] v,
//                Kp[jk] += g D[il] v.
// With the canonical list (i>=j, k>=l, ij>=kl) and g = (i!=j?2:1)(k!=l?2:1)(ij!=kl?2:1),
// J = (Jp + Jp^T)/4 and K = (Kp + Kp^T)/8.  Jp, Kp are accumulated (nfun^2, col-major).
void qbo_jk_list(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                 const double* w, int64_t nq, const int* quartets, const double* g, const double* D, double* Jp,
                 double* Kp, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    jk_list<double>(Basis{nfun, fp, cen, ijk, alpha, w}, nq, quartets, g, D, Jp, Kp);
}
void qbo_jk_list_q(int nfun, const int* fp, const double* cen, const int* ijk, const double* alpha,
                   const double* w, int64_t nq, const int* quartets, const double* g, const double* D, double* Jp,
                   double* Kp, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    jk_list<quad>(Basis{nfun, fp, cen, ijk, alpha, w}, nq, quartets, g, D, Jp, Kp);
}

int qbo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
