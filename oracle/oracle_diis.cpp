// ORACLE — test infrastructure only.
//
// CPU restatement of the DIIS coefficient solvers of Quiqbox.jl v0.6.3 that
// live in third-party packages absent from the reference tree:
//
//  * the objective genxDIISf / genxDIIS∇f (src/HartreeFock.jl:1398-1412) with
//    shiftLastEle! (src/Tools.jl:561-573), which normalises c by its sum and
//    nudges the last entry when the sum is below getAtolVal(Float64) = 4e-16;
//  * LBFGSBsolver! (src/HartreeFock.jl:1416-1430), the reference's default
//    (`defaultDIISsolver = :LBFGS`, :17).  It calls LBFGSB.jl 0.4.1, a wrapper of
//    the Fortran L-BFGS-B 3.0 code, with m = min(getAtolDigits, 50) = 15,
//    factr = 1e5, pgtol = 1e-15, maxfun = maxiter = 10000 and lb = 0 for
//    EDIIS/ADIIS (no bounds for DIIS).  Restated here from the published method:
//    R. H. Byrd, P. Lu, J. Nocedal, C. Zhu, "A limited memory algorithm for bound
//    constrained optimization", SIAM J. Sci. Comput. 16 (1995) 1190-1208 (compact
//    limited-memory matrix, generalised Cauchy point, direct primal subspace
//    minimisation); C. Zhu, R. H. Byrd, P. Lu, J. Nocedal, ACM TOMS 23 (1997)
//    550-560 (Algorithm 778: the stopping tests, memory refresh on a singular or
//    indefinite middle matrix, the L-BFGS update skip rule); J. L. Morales,
//    J. Nocedal, ACM TOMS 38 (2011) 7 (version 3.0: projection of the subspace
//    step with a backtracking fallback); and the line search of J. J. Moré,
//    D. J. Thuente, ACM TOMS 20 (1994) 286-307 (ftol 1e-3, gtol 0.9, xtol 0.1,
//    at most 20 trial steps per search);
//  * SPGBsolver! (src/HartreeFock.jl:1432-1443) through SPGBox.jl 0.7.2:
//    the nonmonotone spectral projected gradient method SPG2 of E. G. Birgin,
//    J. M. Martínez, M. Raydan, SIAM J. Optim. 10 (2000) 1196-1211, with memory
//    m = 20, eps = 1e-15 on the sup-norm of the projected gradient and
//    nitmax = nfevalmax = 10000.
//
// The objective evaluations mutate the iterate exactly as the reference's
// closures do (shiftLastEle! works in place on the vector the optimiser owns).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <vector>

namespace {

constexpr double kEps = 2.220446049250313e-16;   // epsilon(Float64)
constexpr double kShift = 4e-16;                   // getAtolVal(Float64) (src/Arithmetic.jl:42)

using Vec = std::vector<double>;

double dot(const Vec& a, const Vec& b) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

// ---------------------------------------------------------------------------
// Objective (HartreeFock.jl:1398-1412).
struct DiisObjective {
    int n;
    const double* v;   // n
    const double* B;   // n x n, column-major

    // shiftLastEle! (Tools.jl:561-573)
    static double shifted_sum(Vec& c) {
        double s = 0.0;
        for (double x : c) s += x;
        if (s < kShift) {
            const double sh = (s < 0 ? -1.0 : 1.0) * kShift;
            s += sh;
            c.back() += sh;
        }
        return s;
    }
    void parts(const Vec& c, double& vc, double& cBc) const {
        vc = 0.0;
        cBc = 0.0;
        for (int j = 0; j < n; ++j) {
            vc += v[j] * c[j];
            double t = 0.0;
            for (int i = 0; i < n; ++i) t += c[i] * B[i + size_t(n) * j];
            cBc += t * c[j];
        }
    }
    double f(Vec& c) const {
        const double s = shifted_sum(c);
        double vc, cBc;
        parts(c, vc, cBc);
        return vc / s + cBc / (2 * s * s);
    }
    void g(Vec& c, Vec& out) const {
        const double s = shifted_sum(c);
        double vc, cBc;
        parts(c, vc, cBc);
        const double common = vc / (s * s) + cBc / (s * s * s);
        out.assign(n, 0.0);
        for (int i = 0; i < n; ++i) {
            double bc = 0.0;
            for (int j = 0; j < n; ++j) bc += (B[i + size_t(n) * j] + B[j + size_t(n) * i]) * c[j];
            out[i] = v[i] / s + bc / (2 * s * s) - common;
        }
    }
};

// ---------------------------------------------------------------------------
// Small dense helpers.  Upper-triangular matrices are stored column-major with
// leading dimension ld.

// Cholesky A = R^T R of the leading k x k block (upper R in place); returns 0 or
// the 1-based column at which a non-positive pivot appeared.
int chol_upper(double* a, int ld, int k) {
    for (int j = 0; j < k; ++j) {
        double s = 0.0;
        for (int p = 0; p < j; ++p) {
            double t = a[p + ld * j];
            for (int q = 0; q < p; ++q) t -= a[q + ld * p] * a[q + ld * j];
            t /= a[p + ld * p];
            a[p + ld * j] = t;
            s += t * t;
        }
        s = a[j + ld * j] - s;
        if (s <= 0.0) return j + 1;
        a[j + ld * j] = std::sqrt(s);
    }
    return 0;
}

// Solve R^T x = b (trans = true) or R x = b with R upper k x k; returns nonzero on a zero pivot.
int tri_solve(const double* r, int ld, int k, double* b, bool trans) {
    for (int i = 0; i < k; ++i)
        if (r[i + ld * i] == 0.0) return i + 1;
    if (trans) {
        for (int i = 0; i < k; ++i) {
            double t = b[i];
            for (int p = 0; p < i; ++p) t -= r[p + ld * i] * b[p];
            b[i] = t / r[i + ld * i];
        }
    } else {
        for (int i = k - 1; i >= 0; --i) {
            double t = b[i];
            for (int p = i + 1; p < k; ++p) t -= r[i + ld * p] * b[p];
            b[i] = t / r[i + ld * i];
        }
    }
    return 0;
}

// ---------------------------------------------------------------------------
// L-BFGS-B.  Bounds: kind[i] 0 none, 1 lower, 2 both, 3 upper.
class Lbfgsb {
public:
    using FG = std::function<double(Vec&, Vec&)>;   // f(x), gradient into g; may modify x

    Lbfgsb(int n, int m, Vec lo, Vec hi, std::vector<int> kind)
        : n_(n), m_(m), lo_(std::move(lo)), hi_(std::move(hi)), kind_(std::move(kind)) {}

    // Minimise from x (in place); returns the number of iterations.
    int run(Vec& x, const FG& fg, double factr, double pgtol, int maxiter, int maxfun) {
        const double tol = factr * kEps;
        ws_.assign(size_t(n_) * m_, 0.0);
        wy_.assign(size_t(n_) * m_, 0.0);
        sy_.assign(size_t(m_) * m_, 0.0);
        ss_.assign(size_t(m_) * m_, 0.0);
        wt_.assign(size_t(m_) * m_, 0.0);
        where_.assign(n_, 0);
        free_.clear();
        refresh();
        project_initial(x);
        Vec g(n_), z(n_), d(n_), r(n_), t(n_), cw(2 * m_, 0.0), xsave(n_), gsave(n_);
        double f = fg(x, g);
        int nfgv = 1, iter = 0;
        if (proj_grad_norm(x, g) <= pgtol) return iter;
        while (true) {
            // --- search direction: generalised Cauchy point + subspace minimisation
            if (!constrained_ && col_ > 0) {
                z = x;
            } else {
                if (cauchy(x, g, z, cw) != 0) { refresh(); continue; }
                collect_free();
            }
            if (!free_.empty() && col_ > 0) {
                if (form_k() != 0) { refresh(); continue; }
                if (reduced_gradient(x, g, z, cw, r) != 0) { refresh(); continue; }
                if (subspace_min(x, g, z, r) != 0) { refresh(); continue; }
            }
            for (int i = 0; i < n_; ++i) d[i] = z[i] - x[i];
            // --- line search (Moré–Thuente), at most 20 trial steps
            const double dtd = dot(d, d), dnorm = std::sqrt(dtd);
            double stpmx = 1e10;
            if (constrained_) {
                if (iter == 0) {
                    stpmx = 1.0;
                } else {
                    for (int i = 0; i < n_; ++i) {
                        const double a1 = d[i];
                        if (kind_[i] == 0) continue;
                        if (a1 < 0 && kind_[i] <= 2) {
                            const double a2 = lo_[i] - x[i];
                            if (a2 >= 0) stpmx = 0;
                            else if (a1 * stpmx < a2) stpmx = a2 / a1;
                        } else if (a1 > 0 && kind_[i] >= 2) {
                            const double a2 = hi_[i] - x[i];
                            if (a2 <= 0) stpmx = 0;
                            else if (a1 * stpmx > a2) stpmx = a2 / a1;
                        }
                    }
                }
            }
            double stp = (iter == 0 && !boxed_) ? std::min(1.0 / dnorm, stpmx) : 1.0;
            xsave = x;
            gsave = g;
            const double fold = f;
            int ifun = 0, iback = 0;
            double gd = 0, gdold = 0;
            LineSearch ls;
            bool newx = false;
            while (true) {
                gd = dot(g, d);
                if (ifun == 0) {
                    gdold = gd;
                    if (gd >= 0) break;   // not a descent direction
                }
                const int st = ls.step(f, gd, stp, 1e-3, 0.9, 0.1, 0.0, stpmx);
                if (st == LineSearch::kFG) {
                    ++ifun;
                    ++nfgv;
                    iback = ifun - 1;
                    if (stp == 1.0) x = z;
                    else
                        for (int i = 0; i < n_; ++i) x[i] = stp * d[i] + xsave[i];
                    if (iback >= 20) break;
                    f = fg(x, g);
                    continue;
                }
                newx = true;
                break;
            }
            if (!newx) {   // line search failed: back to the previous iterate
                x = xsave;
                g = gsave;
                f = fold;
                if (col_ == 0) return iter + 1;   // abnormal termination
                refresh();
                continue;
            }
            ++iter;
            const double sbgnrm = proj_grad_norm(x, g);
            if (iter >= maxiter || nfgv >= maxfun) return iter;
            if (sbgnrm <= pgtol) return iter;
            const double ddum0 = std::max({std::fabs(fold), std::fabs(f), 1.0});
            if (fold - f <= tol * ddum0) return iter;
            // --- L-BFGS update with s = stp d, y = g - g_old
            for (int i = 0; i < n_; ++i) r[i] = g[i] - gsave[i];
            const double rr = dot(r, r);
            double dr, ddum;
            if (stp == 1.0) {
                dr = gd - gdold;
                ddum = -gdold;
            } else {
                dr = (gd - gdold) * stp;
                for (int i = 0; i < n_; ++i) d[i] *= stp;
                ddum = -gdold * stp;
            }
            if (dr <= kEps * ddum) {   // skip the update
                updated_ = false;
                continue;
            }
            updated_ = true;
            ++iupdat_;
            update_memory(d, r, rr, dr, stp, dtd);
            if (form_t() != 0) { refresh(); continue; }
        }
    }

private:
    // Moré–Thuente line search with its safeguarded cubic/quadratic step.
    struct LineSearch {
        enum { kFG = 0, kConv = 1, kWarn = 2 };
        bool started = false, brackt = false;
        int stage = 1;
        double finit = 0, ginit = 0, gtest = 0, width = 0, width1 = 0;
        double stx = 0, fx = 0, gx = 0, sty = 0, fy = 0, gy = 0, stmin = 0, stmax = 0;

        int step(double f, double g, double& stp, double ftol, double gtol, double xtol, double stpmin,
                 double stpmax) {
            const double xtrapl = 1.1, xtrapu = 4.0;
            if (!started) {
                started = true;
                brackt = false;
                stage = 1;
                finit = f;
                ginit = g;
                gtest = ftol * ginit;
                width = stpmax - stpmin;
                width1 = width / 0.5;
                stx = 0; fx = finit; gx = ginit;
                sty = 0; fy = finit; gy = ginit;
                stmin = 0;
                stmax = stp + xtrapu * stp;
                return kFG;
            }
            const double ftest = finit + stp * gtest;
            if (stage == 1 && f <= ftest && g >= 0) stage = 2;
            int task = kFG;
            if (brackt && (stp <= stmin || stp >= stmax)) task = kWarn;
            if (brackt && stmax - stmin <= xtol * stmax) task = kWarn;
            if (stp == stpmax && f <= ftest && g <= gtest) task = kWarn;
            if (stp == stpmin && (f > ftest || g >= gtest)) task = kWarn;
            if (f <= ftest && std::fabs(g) <= gtol * (-ginit)) task = kConv;
            if (task != kFG) return task;
            if (stage == 1 && f <= fx && f > ftest) {
                // modified function psi(stp) = f - stp * gtest in the first stage
                double fm = f - stp * gtest, fxm = fx - stx * gtest, fym = fy - sty * gtest;
                double gm = g - gtest, gxm = gx - gtest, gym = gy - gtest;
                cstep(stx, fxm, gxm, sty, fym, gym, stp, fm, gm, brackt, stmin, stmax);
                fx = fxm + stx * gtest;
                fy = fym + sty * gtest;
                gx = gxm + gtest;
                gy = gym + gtest;
            } else {
                cstep(stx, fx, gx, sty, fy, gy, stp, f, g, brackt, stmin, stmax);
            }
            if (brackt) {
                if (std::fabs(sty - stx) >= 0.66 * width1) stp = stx + 0.5 * (sty - stx);
                width1 = width;
                width = std::fabs(sty - stx);
            }
            if (brackt) {
                stmin = std::min(stx, sty);
                stmax = std::max(stx, sty);
            } else {
                stmin = stp + xtrapl * (stp - stx);
                stmax = stp + xtrapu * (stp - stx);
            }
            stp = std::max(stp, stpmin);
            stp = std::min(stp, stpmax);
            if ((brackt && (stp <= stmin || stp >= stmax)) || (brackt && stmax - stmin <= xtol * stmax)) stp = stx;
            return kFG;
        }

        // Safeguarded step of the interval update (Moré & Thuente 1994, section 4).
        static void cstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp,
                          double fp, double dp, bool& brackt, double stpmin, double stpmax) {
            const double sgnd = dp * (dx / std::fabs(dx));
            double stpf;
            if (fp > fx) {   // higher value: minimiser bracketed
                const double theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
                const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
                double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
                if (stp < stx) gamma = -gamma;
                const double p = (gamma - dx) + theta, q = ((gamma - dx) + gamma) + dp, r = p / q;
                const double stpc = stx + r * (stp - stx);
                const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2) * (stp - stx);
                stpf = (std::fabs(stpc - stx) < std::fabs(stpq - stx)) ? stpc : stpc + (stpq - stpc) / 2;
                brackt = true;
            } else if (sgnd < 0) {   // lower value, derivatives of opposite sign
                const double theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
                const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
                double gamma = s * std::sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
                if (stp > stx) gamma = -gamma;
                const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dx, r = p / q;
                const double stpc = stp + r * (stx - stp);
                const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
                stpf = (std::fabs(stpc - stp) > std::fabs(stpq - stp)) ? stpc : stpq;
                brackt = true;
            } else if (std::fabs(dp) < std::fabs(dx)) {   // same sign, derivative magnitude decreases
                const double theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
                const double s = std::max({std::fabs(theta), std::fabs(dx), std::fabs(dp)});
                double gamma = s * std::sqrt(std::max(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
                if (stp > stx) gamma = -gamma;
                const double p = (gamma - dp) + theta, q = (gamma + (dx - dp)) + gamma, r = p / q;
                double stpc;
                if (r < 0 && gamma != 0) stpc = stp + r * (stx - stp);
                else if (stp > stx) stpc = stpmax;
                else stpc = stpmin;
                const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
                if (brackt) {
                    stpf = (std::fabs(stpc - stp) < std::fabs(stpq - stp)) ? stpc : stpq;
                    if (stp > stx) stpf = std::min(stp + 0.66 * (sty - stp), stpf);
                    else stpf = std::max(stp + 0.66 * (sty - stp), stpf);
                } else {
                    stpf = (std::fabs(stpc - stp) > std::fabs(stpq - stp)) ? stpc : stpq;
                    stpf = std::min(stpmax, stpf);
                    stpf = std::max(stpmin, stpf);
                }
            } else {   // same sign, derivative magnitude does not decrease
                if (brackt) {
                    const double theta = 3 * (fp - fy) / (sty - stp) + dy + dp;
                    const double s = std::max({std::fabs(theta), std::fabs(dy), std::fabs(dp)});
                    double gamma = s * std::sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
                    if (stp > sty) gamma = -gamma;
                    const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dy, r = p / q;
                    stpf = stp + r * (sty - stp);
                } else if (stp > stx) {
                    stpf = stpmax;
                } else {
                    stpf = stpmin;
                }
            }
            if (fp > fx) {
                sty = stp; fy = fp; dy = dp;
            } else {
                if (sgnd < 0) { sty = stx; fy = fx; dy = dx; }
                stx = stp; fx = fp; dx = dp;
            }
            stp = stpf;
        }
    };

    void refresh() {
        col_ = 0;
        head_ = 0;
        tail_ = 0;
        theta_ = 1.0;
        iupdat_ = 0;
        updated_ = false;
    }

    int slot(int k) const { return (head_ + k) % m_; }   // k-th stored pair, oldest first
    double& WS(int i, int k) { return ws_[i + size_t(n_) * slot(k)]; }
    double& WY(int i, int k) { return wy_[i + size_t(n_) * slot(k)]; }
    double& SY(int i, int j) { return sy_[i + size_t(m_) * j]; }
    double& SS(int i, int j) { return ss_[i + size_t(m_) * j]; }

    // Project x0 into the box; record which variables are bounded.
    void project_initial(Vec& x) {
        constrained_ = false;
        boxed_ = true;
        for (int i = 0; i < n_; ++i) {
            if (kind_[i] > 0) {
                if (kind_[i] <= 2 && x[i] <= lo_[i]) x[i] = std::max(x[i], lo_[i]);
                else if (kind_[i] >= 2 && x[i] >= hi_[i]) x[i] = std::min(x[i], hi_[i]);
            }
        }
        for (int i = 0; i < n_; ++i) {
            if (kind_[i] != 2) boxed_ = false;
            if (kind_[i] == 0) {
                where_[i] = -1;
            } else {
                constrained_ = true;
                where_[i] = (kind_[i] == 2 && hi_[i] - lo_[i] <= 0) ? 3 : 0;
            }
        }
    }

    double proj_grad_norm(const Vec& x, const Vec& g) const {
        double s = 0.0;
        for (int i = 0; i < n_; ++i) {
            double gi = g[i];
            if (kind_[i] != 0) {
                if (gi < 0) {
                    if (kind_[i] >= 2) gi = std::max(x[i] - hi_[i], gi);
                } else {
                    if (kind_[i] <= 2) gi = std::min(x[i] - lo_[i], gi);
                }
            }
            s = std::max(s, std::fabs(gi));
        }
        return s;
    }

    // p = M v for the 2col middle matrix M of the compact form B = theta I - W M W^T,
    // W = [Y, theta S], through the factorisation of T = theta S'S + L D^-1 L^T (wt_).
    int middle_product(const double* v, double* p) {
        const int col = col_;
        if (col == 0) return 0;
        p[col] = v[col];
        for (int i = 1; i < col; ++i) {
            double sum = 0.0;
            for (int k = 0; k < i; ++k) sum += SY(i, k) * v[k] / SY(k, k);
            p[col + i] = v[col + i] + sum;
        }
        if (tri_solve(wt_.data(), m_, col, p + col, true)) return -1;
        for (int i = 0; i < col; ++i) p[i] = v[i] / std::sqrt(SY(i, i));
        if (tri_solve(wt_.data(), m_, col, p + col, false)) return -1;
        for (int i = 0; i < col; ++i) p[i] = -p[i] / std::sqrt(SY(i, i));
        for (int i = 0; i < col; ++i) {
            double sum = 0.0;
            for (int k = i + 1; k < col; ++k) sum += SY(k, i) * p[col + k] / SY(i, i);
            p[i] += sum;
        }
        return 0;
    }

    // Binary min-heap over t[0..cnt) with payload ord; build = true builds it from scratch.
    // On return the least element sits at t[cnt-1] and t[0..cnt-1) is a heap again.
    static void heap_pop(int cnt, double* t, int* ord, bool build) {
        if (build) {
            for (int k = 1; k < cnt; ++k) {
                const double val = t[k];
                const int idx = ord[k];
                int i = k;
                while (i > 0) {
                    const int j = (i + 1) / 2 - 1;
                    if (val < t[j]) {
                        t[i] = t[j];
                        ord[i] = ord[j];
                        i = j;
                    } else {
                        break;
                    }
                }
                t[i] = val;
                ord[i] = idx;
            }
        }
        if (cnt > 1) {
            const double out = t[0];
            const int oidx = ord[0];
            const double val = t[cnt - 1];
            const int idx = ord[cnt - 1];
            int i = 0;   // 1-based position i+1; children 2(i+1), 2(i+1)+1
            while (true) {
                int j = 2 * (i + 1) - 1;
                if (j <= cnt - 2) {   // the sibling j + 1 may be the slot of the re-inserted value
                    if (t[j + 1] < t[j]) j = j + 1;
                    if (t[j] < val) {
                        t[i] = t[j];
                        ord[i] = ord[j];
                        i = j;
                        continue;
                    }
                }
                break;
            }
            t[i] = val;
            ord[i] = idx;
            t[cnt - 1] = out;
            ord[cnt - 1] = oidx;
        }
    }

    // Generalised Cauchy point of the quadratic model along the projected
    // steepest-descent path (Byrd et al. 1995, section 4).  xcp and
    // c = W^T (xcp - x) are the outputs; where_ is updated.
    int cauchy(const Vec& x, const Vec& g, Vec& xcp, Vec& c) {
        const int col = col_, col2 = 2 * col_;
        if (proj_grad_norm(x, g) <= 0.0) {
            xcp = x;
            return 0;
        }
        bool bnded = true;
        int nfree = n_, nbreak = 0, ibkmin = 0;
        double bkmin = 0.0, f1 = 0.0;
        std::vector<double> tbrk(n_), d(n_);
        std::vector<int> ord(n_);
        Vec p(col2, 0.0), v(col2, 0.0), wbp(col2, 0.0);
        double tl = 0.0, tu = 0.0;
        for (int i = 0; i < n_; ++i) {
            const double neggi = -g[i];
            if (where_[i] != 3 && where_[i] != -1) {
                if (kind_[i] <= 2) tl = x[i] - lo_[i];
                if (kind_[i] >= 2) tu = hi_[i] - x[i];
                const bool xlower = kind_[i] <= 2 && tl <= 0;
                const bool xupper = kind_[i] >= 2 && tu <= 0;
                where_[i] = 0;
                if (xlower) {
                    if (neggi <= 0) where_[i] = 1;
                } else if (xupper) {
                    if (neggi >= 0) where_[i] = 2;
                } else {
                    if (std::fabs(neggi) <= 0) where_[i] = -3;
                }
            }
            if (where_[i] != 0 && where_[i] != -1) {
                d[i] = 0.0;
            } else {
                d[i] = neggi;
                f1 -= neggi * neggi;
                for (int j = 0; j < col; ++j) {
                    p[j] += WY(i, j) * neggi;
                    p[col + j] += WS(i, j) * neggi;
                }
                if (kind_[i] <= 2 && kind_[i] != 0 && neggi < 0) {
                    ord[nbreak] = i;
                    tbrk[nbreak] = tl / (-neggi);
                    if (nbreak == 0 || tbrk[nbreak] < bkmin) { bkmin = tbrk[nbreak]; ibkmin = nbreak; }
                    ++nbreak;
                } else if (kind_[i] >= 2 && neggi > 0) {
                    ord[nbreak] = i;
                    tbrk[nbreak] = tu / neggi;
                    if (nbreak == 0 || tbrk[nbreak] < bkmin) { bkmin = tbrk[nbreak]; ibkmin = nbreak; }
                    ++nbreak;
                } else {
                    --nfree;
                    ord[nfree] = i;
                    if (std::fabs(neggi) > 0) bnded = false;
                }
            }
        }
        if (theta_ != 1.0)
            for (int j = 0; j < col; ++j) p[col + j] *= theta_;
        xcp = x;
        if (nbreak == 0 && nfree == n_) return 0;   // d = 0
        c.assign(2 * m_, 0.0);
        double f2 = -theta_ * f1;
        const double f2_org = f2;
        if (col > 0) {
            if (middle_product(p.data(), v.data())) return -1;
            double pv = 0.0;
            for (int j = 0; j < col2; ++j) pv += v[j] * p[j];
            f2 -= pv;
        }
        double dtm = -f1 / f2, tsum = 0.0;
        if (nbreak > 0) {
            int nleft = nbreak, it = 1;
            double tj = 0.0;
            bool done = false, allfixed = false;
            while (!done) {
                const double tj0 = tj;
                int ibp;
                if (it == 1) {
                    tj = bkmin;
                    ibp = ord[ibkmin];
                } else {
                    if (it == 2 && ibkmin != nbreak - 1) {
                        tbrk[ibkmin] = tbrk[nbreak - 1];
                        ord[ibkmin] = ord[nbreak - 1];
                    }
                    heap_pop(nleft, tbrk.data(), ord.data(), it == 2);
                    tj = tbrk[nleft - 1];
                    ibp = ord[nleft - 1];
                }
                const double dt = tj - tj0;
                if (dtm < dt) break;
                tsum += dt;
                --nleft;
                ++it;
                const double dibp = d[ibp];
                d[ibp] = 0.0;
                double zibp;
                if (dibp > 0) {
                    zibp = hi_[ibp] - x[ibp];
                    xcp[ibp] = hi_[ibp];
                    where_[ibp] = 2;
                } else {
                    zibp = lo_[ibp] - x[ibp];
                    xcp[ibp] = lo_[ibp];
                    where_[ibp] = 1;
                }
                if (nleft == 0 && nbreak == n_) {   // every variable fixed
                    dtm = dt;
                    allfixed = true;
                    break;
                }
                const double dibp2 = dibp * dibp;
                f1 = f1 + dt * f2 + dibp2 - theta_ * dibp * zibp;
                f2 = f2 - theta_ * dibp2;
                if (col > 0) {
                    for (int j = 0; j < col2; ++j) c[j] += dt * p[j];
                    for (int j = 0; j < col; ++j) {
                        wbp[j] = WY(ibp, j);
                        wbp[col + j] = theta_ * WS(ibp, j);
                    }
                    if (middle_product(wbp.data(), v.data())) return -1;
                    double wmc = 0, wmp = 0, wmw = 0;
                    for (int j = 0; j < col2; ++j) {
                        wmc += c[j] * v[j];
                        wmp += p[j] * v[j];
                        wmw += wbp[j] * v[j];
                    }
                    for (int j = 0; j < col2; ++j) p[j] -= dibp * wbp[j];
                    f1 += dibp * wmc;
                    f2 += 2.0 * dibp * wmp - dibp2 * wmw;
                }
                f2 = std::max(kEps * f2_org, f2);
                if (nleft > 0) {
                    dtm = -f1 / f2;
                } else if (bnded) {
                    f1 = 0;
                    f2 = 0;
                    dtm = 0;
                    done = true;
                } else {
                    dtm = -f1 / f2;
                    done = true;
                }
            }
            if (allfixed) {
                if (col > 0)
                    for (int j = 0; j < col2; ++j) c[j] += dtm * p[j];
                return 0;
            }
        }
        if (dtm <= 0) dtm = 0;
        tsum += dtm;
        for (int i = 0; i < n_; ++i) xcp[i] += tsum * d[i];
        if (col > 0)
            for (int j = 0; j < col2; ++j) c[j] += dtm * p[j];
        return 0;
    }

    void collect_free() {
        free_.clear();
        active_.clear();
        for (int i = 0; i < n_; ++i) (where_[i] <= 0 ? free_ : active_).push_back(i);
    }

    // LEL^T factorisation of the indefinite middle matrix of the reduced problem,
    //   K = [-D - Y'ZZ'Y/theta   L_a' - R_z' ; L_a - R_z   theta S'AA'S],
    // stored as the upper factor wn_ (2col x 2col, leading dimension 2m).
    int form_k() {
        const int col = col_, m2 = 2 * m_;
        wn_.assign(size_t(m2) * m2, 0.0);
        auto WN = [&](int i, int j) -> double& { return wn_[i + size_t(m2) * j]; };
        for (int iy = 0; iy < col; ++iy)
            for (int jy = 0; jy <= iy; ++jy) {
                double yzzy = 0, saas = 0;
                for (int k : free_) yzzy += WY(k, iy) * WY(k, jy);
                for (int k : active_) saas += WS(k, iy) * WS(k, jy);
                WN(jy, iy) = yzzy / theta_;
                WN(col + jy, col + iy) = saas * theta_;
            }
        for (int iy = 0; iy < col; ++iy) {
            WN(iy, iy) += SY(iy, iy);
            for (int jy = 0; jy < col; ++jy) {
                double val = 0;
                if (jy < iy) {   // -L_a(iy, jy): s_iy' A A' y_jy
                    for (int k : active_) val += WS(k, iy) * WY(k, jy);
                    val = -val;
                } else {         // R_z(iy, jy): s_iy' Z Z' y_jy
                    for (int k : free_) val += WS(k, iy) * WY(k, jy);
                }
                WN(jy, col + iy) = val;
            }
        }
        if (chol_upper(wn_.data(), m2, col)) return -1;
        for (int js = col; js < 2 * col; ++js)
            if (tri_solve(wn_.data(), m2, col, &WN(0, js), true)) return -1;
        for (int is = col; is < 2 * col; ++is)
            for (int js = is; js < 2 * col; ++js) {
                double s = 0;
                for (int k = 0; k < col; ++k) s += WN(k, is) * WN(k, js);
                WN(is, js) += s;
            }
        if (chol_upper(&WN(col, col), m2, col)) return -2;
        return 0;
    }

    // T = theta S'S + L D^-1 L^T, Cholesky factor into wt_.
    int form_t() {
        const int col = col_;
        for (int j = 0; j < col; ++j) wt_[0 + size_t(m_) * j] = theta_ * SS(0, j);
        for (int i = 1; i < col; ++i)
            for (int j = i; j < col; ++j) {
                const int k1 = std::min(i, j);
                double s = 0;
                for (int k = 0; k < k1; ++k) s += SY(i, k) * SY(j, k) / SY(k, k);
                wt_[i + size_t(m_) * j] = s + theta_ * SS(i, j);
            }
        return chol_upper(wt_.data(), m_, col) ? -3 : 0;
    }

    // r = -Z^T (B (xcp - x) + g) over the free variables.
    int reduced_gradient(const Vec& x, const Vec& g, const Vec& z, const Vec& c, Vec& r) {
        const int col = col_;
        r.assign(free_.size(), 0.0);
        if (!constrained_ && col > 0) {
            for (int i = 0; i < n_; ++i) r[i] = -g[i];
            return 0;
        }
        for (size_t q = 0; q < free_.size(); ++q) {
            const int k = free_[q];
            r[q] = -theta_ * (z[k] - x[k]) - g[k];
        }
        Vec a(2 * m_, 0.0);
        if (middle_product(c.data(), a.data())) return -8;
        for (int j = 0; j < col; ++j) {
            const double a1 = a[j], a2 = theta_ * a[col + j];
            for (size_t q = 0; q < free_.size(); ++q) {
                const int k = free_[q];
                r[q] += WY(k, j) * a1 + WS(k, j) * a2;
            }
        }
        return 0;
    }

    // Direct primal subspace minimisation from the Cauchy point, then projection
    // of the Newton point onto the box with a backtracking fallback (version 3.0).
    int subspace_min(const Vec& xx, const Vec& gg, Vec& x, Vec& d) {
        const int col = col_, m2 = 2 * m_, nsub = (int)free_.size();
        Vec wv(2 * col, 0.0);
        for (int i = 0; i < col; ++i) {
            double t1 = 0, t2 = 0;
            for (int j = 0; j < nsub; ++j) {
                const int k = free_[j];
                t1 += WY(k, i) * d[j];
                t2 += WS(k, i) * d[j];
            }
            wv[i] = t1;
            wv[col + i] = theta_ * t2;
        }
        // the factor spans the leading 2col x 2col block of wn_ (leading dimension 2m)
        if (tri_solve(wn_.data(), m2, 2 * col, wv.data(), true)) return -1;
        for (int i = 0; i < col; ++i) wv[i] = -wv[i];
        if (tri_solve(wn_.data(), m2, 2 * col, wv.data(), false)) return -1;
        for (int jy = 0; jy < col; ++jy)
            for (int i = 0; i < nsub; ++i) {
                const int k = free_[i];
                d[i] += WY(k, jy) * wv[jy] / theta_ + WS(k, jy) * wv[col + jy];
            }
        for (int i = 0; i < nsub; ++i) d[i] /= theta_;
        // projection of x + d
        Vec xp = x;
        bool hit = false;
        for (int i = 0; i < nsub; ++i) {
            const int k = free_[i];
            const double dk = d[i], xk = x[k];
            if (kind_[k] == 0) {
                x[k] = xk + dk;
            } else if (kind_[k] == 1) {
                x[k] = std::max(lo_[k], xk + dk);
                if (x[k] == lo_[k]) hit = true;
            } else if (kind_[k] == 2) {
                x[k] = std::min(hi_[k], std::max(lo_[k], xk + dk));
                if (x[k] == lo_[k] || x[k] == hi_[k]) hit = true;
            } else {
                x[k] = std::min(hi_[k], xk + dk);
                if (x[k] == hi_[k]) hit = true;
            }
        }
        if (!hit) return 0;
        double ddp = 0;
        for (int i = 0; i < n_; ++i) ddp += (x[i] - xx[i]) * gg[i];
        if (ddp <= 0) return 0;
        // positive directional derivative after projection: backtrack along d instead
        x = xp;
        double alpha = 1.0, temp1 = alpha;
        int ibd = -1;
        for (int i = 0; i < nsub; ++i) {
            const int k = free_[i];
            const double dk = d[i];
            if (kind_[k] == 0) continue;
            if (dk < 0 && kind_[k] <= 2) {
                const double t2 = lo_[k] - x[k];
                if (t2 >= 0) temp1 = 0;
                else if (dk * alpha < t2) temp1 = t2 / dk;
            } else if (dk > 0 && kind_[k] >= 2) {
                const double t2 = hi_[k] - x[k];
                if (t2 <= 0) temp1 = 0;
                else if (dk * alpha > t2) temp1 = t2 / dk;
            }
            if (temp1 < alpha) {
                alpha = temp1;
                ibd = i;
            }
        }
        if (alpha < 1.0 && ibd >= 0) {
            const double dk = d[ibd];
            const int k = free_[ibd];
            if (dk > 0) {
                x[k] = hi_[k];
                d[ibd] = 0;
            } else if (dk < 0) {
                x[k] = lo_[k];
                d[ibd] = 0;
            }
        }
        for (int i = 0; i < nsub; ++i) x[free_[i]] += alpha * d[i];
        return 0;
    }

    // Append the pair (s, y) to the limited memory and the inner-product matrices.
    void update_memory(const Vec& s, const Vec& y, double rr, double dr, double stp, double dtd) {
        if (iupdat_ <= m_) {
            col_ = iupdat_;
            tail_ = (head_ + iupdat_ - 1) % m_;
        } else {
            tail_ = (tail_ + 1) % m_;
            head_ = (head_ + 1) % m_;
        }
        for (int i = 0; i < n_; ++i) {
            ws_[i + size_t(n_) * tail_] = s[i];
            wy_[i + size_t(n_) * tail_] = y[i];
        }
        theta_ = rr / dr;
        const int col = col_;
        if (iupdat_ > m_) {   // drop the oldest pair from SS (upper) and SY (lower)
            for (int j = 0; j < col - 1; ++j) {
                for (int i = 0; i <= j; ++i) SS(i, j) = SS(i + 1, j + 1);
                for (int i = j; i < col - 1; ++i) SY(i, j) = SY(i + 1, j + 1);
            }
        }
        for (int j = 0; j < col - 1; ++j) {
            double a = 0, b = 0;
            for (int i = 0; i < n_; ++i) {
                a += s[i] * WY(i, j);
                b += WS(i, j) * s[i];
            }
            SY(col - 1, j) = a;
            SS(j, col - 1) = b;
        }
        SS(col - 1, col - 1) = (stp == 1.0) ? dtd : stp * stp * dtd;
        SY(col - 1, col - 1) = dr;
    }

    int n_, m_;
    Vec lo_, hi_;
    std::vector<int> kind_;
    Vec ws_, wy_, sy_, ss_, wt_, wn_;
    std::vector<int> where_, free_, active_;
    int col_ = 0, head_ = 0, tail_ = 0, iupdat_ = 0;
    double theta_ = 1.0;
    bool updated_ = false, constrained_ = false, boxed_ = false;
};

// ---------------------------------------------------------------------------
// SPG2 (Birgin, Martínez & Raydan 2000) with lower bounds lb (or none).
int spg(Vec& x, const std::function<double(Vec&)>& f, const std::function<void(Vec&, Vec&)>& g, bool bounded,
        double lb, double eps, int nitmax, int nfevalmax, int mem) {
    const int n = (int)x.size();
    const double lmin = 1e-30, lmax = 1e30, gamma = 1e-4, sigma1 = 0.1, sigma2 = 0.9;
    auto project = [&](Vec& y) {
        if (bounded)
            for (double& t : y) t = std::max(t, lb);
    };
    auto pg_norm = [&](const Vec& xv, const Vec& gv) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) {
            double t = xv[i] - gv[i];
            if (bounded) t = std::max(t, lb);
            s = std::max(s, std::fabs(t - xv[i]));
        }
        return s;
    };
    project(x);
    Vec gr(n), xn(n), gn(n), dv(n);
    double fc = f(x);
    g(x, gr);
    int nfeval = 1, nit = 0;
    double gnorm = pg_norm(x, gr);
    if (gnorm <= eps) return 0;
    Vec fprev(mem, fc);
    double lam = std::min(lmax, std::max(lmin, 1.0 / gnorm));
    while (nit < nitmax) {
        for (int i = 0; i < n; ++i) xn[i] = x[i] - lam * gr[i];
        project(xn);
        for (int i = 0; i < n; ++i) dv[i] = xn[i] - x[i];
        const double gtd = dot(gr, dv);
        const double fref = *std::max_element(fprev.begin(), fprev.end());
        double alpha = 1.0;
        for (int i = 0; i < n; ++i) xn[i] = x[i] + alpha * dv[i];
        double fn = f(xn);
        ++nfeval;
        while (fn > fref + gamma * alpha * gtd) {
            const double atemp = -0.5 * gtd * alpha * alpha / (fn - fc - alpha * gtd);
            if (atemp >= sigma1 && atemp <= sigma2 * alpha) alpha = atemp;
            else alpha /= 2;
            for (int i = 0; i < n; ++i) xn[i] = x[i] + alpha * dv[i];
            fn = f(xn);
            if (++nfeval > nfevalmax) {
                x = xn;
                return 2;
            }
        }
        ++nit;
        fprev[nit % mem] = fn;
        g(xn, gn);
        double sts = 0, sty = 0;
        for (int i = 0; i < n; ++i) {
            const double s = xn[i] - x[i], y = gn[i] - gr[i];
            sts += s * s;
            sty += s * y;
        }
        lam = sty <= 0 ? lmax : std::min(lmax, std::max(lmin, sts / sty));
        x = xn;
        gr = gn;
        fc = fn;
        gnorm = pg_norm(x, gr);
        if (gnorm <= eps) return 0;
    }
    return 1;
}

}  // namespace

extern "C" {

void qbo_diis_cm(int convex, int n, const double* v, const double* B, double* c);   // oracle_scf.cpp

// DIIS coefficient problem of the reference (constraintSolver!, HartreeFock.jl:1416-1487):
// solver 0 L-BFGS-B (default), 1 SPG, 2 Lagrange multipliers (CMsolver!), on c (length n,
// the starting point on entry and the normalised coefficients on return); convex != 0 adds
// c >= 0 (EDIIS / ADIIS).  Returns the solver's iteration count (L-BFGS-B) or status (SPG).
int qbo_diis_solve_iter(int solver, int convex, int n, const double* v, const double* B, double* c) {
    if (solver == 2) {
        qbo_diis_cm(convex, n, v, B, c);
        return 0;
    }
    DiisObjective obj{n, v, B};
    Vec x(c, c + n);
    int out;
    if (solver == 0) {
        Lbfgsb opt(n, std::min(15, 50), Vec(n, convex ? 0.0 : -INFINITY), Vec(n, INFINITY),
                   std::vector<int>(n, convex ? 1 : 0));
        out = opt.run(x, [&](Vec& xv, Vec& gv) { const double fv = obj.f(xv); obj.g(xv, gv); return fv; }, 1e5,
                      1e-15, 10000, 10000);
    } else {
        out = spg(x, [&](Vec& xv) { return obj.f(xv); }, [&](Vec& xv, Vec& gv) { obj.g(xv, gv); }, convex != 0, 0.0,
                  1e-15, 10000, 10000, 20);
    }
    const double s = DiisObjective::shifted_sum(x);
    for (int i = 0; i < n; ++i) c[i] = x[i] / s;
    return out;
}

}  // extern "C"
