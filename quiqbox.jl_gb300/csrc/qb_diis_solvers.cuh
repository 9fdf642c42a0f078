// DIIS coefficient solvers on the device.
//
// The reference solves, every DIIS / EDIIS / ADIIS step, the small problem
//   minimise f(c) = v.c / s + c^T B c / (2 s^2),   s = sum(c)   [c >= 0 for EDIIS/ADIIS]
// (genxDIISf / genxDIIS∇f, src/HartreeFock.jl:1398-1412; shiftLastEle!, src/Tools.jl:561-573)
// with one of three solvers (constraintSolver!, :1479-1487):
//   QB_DIIS_LBFGS (default, :17)  LBFGSBsolver! (:1416-1430): LBFGSB.jl 0.4.1, i.e. the
//                                 L-BFGS-B 3.0 method, m = 15 corrections, factr = 1e5,
//                                 pgtol = 1e-15, lb = 0 or none;
//   QB_DIIS_SPGB                  SPGBsolver! (:1432-1443): SPGBox.jl 0.7.2, the
//                                 nonmonotone spectral projected gradient (memory 20,
//                                 eps = 1e-15);
//   QB_DIIS_LCM                   CMsolver! (:1445-1477), qb_cm_solve below.
// L-BFGS-B is the method of Byrd, Lu, Nocedal & Zhu (SIAM J. Sci. Comput. 16, 1995) with
// the stopping and memory-refresh rules of Zhu et al. (ACM TOMS Algorithm 778, 1997), the
// projected subspace step of Morales & Nocedal (ACM TOMS 38, 2011) and the line search of
// Moré & Thuente (ACM TOMS 20, 1994); SPG is SPG2 of Birgin, Martínez & Raydan (SIAM J.
// Optim. 10, 2000).
//
// The problems have at most 16 variables, so one thread runs a solve; its state lives in
// a QbDiisWork block in global memory supplied by the caller (about 20 KB), never in the
// thread's local frame.  Every loop is bounded (10000 iterations and evaluations, 20 trial
// steps per line search, as in the reference's settings).  The starting point is c on
// entry (the previous solution with a 1 appended for the newest entry, as the reference's
// per-method coefficient vector carries over); on return c holds the normalised solution.
#pragma once
#include "quiqbox_gb300.h"   // QB_DIIS_LBFGS / QB_DIIS_SPGB / QB_DIIS_LCM

#define QB_DS_N 16   // variables (DIIS subspace size <= 15, plus slack)
#define QB_DS_M 15   // L-BFGS-B corrections: min(getAtolDigits(Float64), 50)

struct QbDiisWork {
    double B[QB_DS_N * QB_DS_N], v[QB_DS_N];
    double ws[QB_DS_N * QB_DS_M], wy[QB_DS_N * QB_DS_M];
    double sy[QB_DS_M * QB_DS_M], ss[QB_DS_M * QB_DS_M], wt[QB_DS_M * QB_DS_M];
    double wn[4 * QB_DS_M * QB_DS_M];
    double x[QB_DS_N], g[QB_DS_N], z[QB_DS_N], d[QB_DS_N], r[QB_DS_N], xs[QB_DS_N], gs[QB_DS_N], xp[QB_DS_N];
    double cw[2 * QB_DS_M], p[2 * QB_DS_M], vv[2 * QB_DS_M], wbp[2 * QB_DS_M], wv[2 * QB_DS_M];
    double tb[QB_DS_N], fprev[20];
    double cmB[QB_DS_N * QB_DS_N], cmA[(QB_DS_N + 1) * (QB_DS_N + 1)], cmW[(QB_DS_N + 1) * (QB_DS_N + 1)];
    double cmb[QB_DS_N + 1], cmx[QB_DS_N + 1];
    int ord[QB_DS_N], where[QB_DS_N], freel[QB_DS_N], actl[QB_DS_N];
    int nfree, nact;
    int iters;   // solver iterations of the last solve (diagnostics)
};

namespace qbds {

constexpr double kEps = 2.220446049250313e-16;
constexpr double kShift = 4e-16;   // getAtolVal(Float64) (src/Arithmetic.jl:42)

// shiftLastEle! on the iterate
__device__ inline double shifted_sum(int n, double* c) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += c[i];
    if (s < kShift) {
        const double sh = (s < 0 ? -1.0 : 1.0) * kShift;
        s += sh;
        c[n - 1] += sh;
    }
    return s;
}

__device__ inline void parts(const QbDiisWork& w, int n, const double* c, double& vc, double& cBc) {
    vc = 0.0;
    cBc = 0.0;
    for (int j = 0; j < n; ++j) {
        vc += w.v[j] * c[j];
        double t = 0.0;
        for (int i = 0; i < n; ++i) t += c[i] * w.B[i + QB_DS_N * j];
        cBc += t * c[j];
    }
}

__device__ inline double obj_f(const QbDiisWork& w, int n, double* c) {
    const double s = shifted_sum(n, c);
    double vc, cBc;
    parts(w, n, c, vc, cBc);
    return vc / s + cBc / (2 * s * s);
}

__device__ inline void obj_g(const QbDiisWork& w, int n, double* c, double* g) {
    const double s = shifted_sum(n, c);
    double vc, cBc;
    parts(w, n, c, vc, cBc);
    const double common = vc / (s * s) + cBc / (s * s * s);
    for (int i = 0; i < n; ++i) {
        double bc = 0.0;
        for (int j = 0; j < n; ++j) bc += (w.B[i + QB_DS_N * j] + w.B[j + QB_DS_N * i]) * c[j];
        g[i] = w.v[i] / s + bc / (2 * s * s) - common;
    }
}

__device__ inline double fg(const QbDiisWork& w, int n, double* c, double* g) {
    const double f = obj_f(w, n, c);
    obj_g(w, n, c, g);
    return f;
}

// Cholesky R^T R of the leading k x k block, upper R in place; nonzero on a non-positive pivot.
__device__ inline int chol_upper(double* a, int ld, int k) {
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
        a[j + ld * j] = sqrt(s);
    }
    return 0;
}

// R^T x = b (trans) or R x = b, R upper k x k in place of b; nonzero on a zero pivot.
__device__ inline int tri_solve(const double* r, int ld, int k, double* b, bool trans) {
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

// Moré–Thuente line search state (one search).
struct Search {
    bool brackt;
    int stage;
    double finit, ginit, gtest, width, width1, stx, fx, gx, sty, fy, gy, stmin, stmax;
};

// Safeguarded step and interval update.
__device__ inline void cstep(double& stx, double& fx, double& dx, double& sty, double& fy, double& dy, double& stp,
                             double fp, double dp, bool& brackt, double stpmin, double stpmax) {
    const double sgnd = dp * (dx / fabs(dx));
    double stpf;
    if (fp > fx) {
        const double theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
        const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
        double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
        if (stp < stx) gamma = -gamma;
        const double p = (gamma - dx) + theta, q = ((gamma - dx) + gamma) + dp, r = p / q;
        const double stpc = stx + r * (stp - stx);
        const double stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2) * (stp - stx);
        stpf = (fabs(stpc - stx) < fabs(stpq - stx)) ? stpc : stpc + (stpq - stpc) / 2;
        brackt = true;
    } else if (sgnd < 0) {
        const double theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
        const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
        double gamma = s * sqrt((theta / s) * (theta / s) - (dx / s) * (dp / s));
        if (stp > stx) gamma = -gamma;
        const double p = (gamma - dp) + theta, q = ((gamma - dp) + gamma) + dx, r = p / q;
        const double stpc = stp + r * (stx - stp);
        const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
        stpf = (fabs(stpc - stp) > fabs(stpq - stp)) ? stpc : stpq;
        brackt = true;
    } else if (fabs(dp) < fabs(dx)) {
        const double theta = 3 * (fx - fp) / (stp - stx) + dx + dp;
        const double s = fmax(fabs(theta), fmax(fabs(dx), fabs(dp)));
        double gamma = s * sqrt(fmax(0.0, (theta / s) * (theta / s) - (dx / s) * (dp / s)));
        if (stp > stx) gamma = -gamma;
        const double p = (gamma - dp) + theta, q = (gamma + (dx - dp)) + gamma, r = p / q;
        double stpc;
        if (r < 0 && gamma != 0) stpc = stp + r * (stx - stp);
        else if (stp > stx) stpc = stpmax;
        else stpc = stpmin;
        const double stpq = stp + (dp / (dp - dx)) * (stx - stp);
        if (brackt) {
            stpf = (fabs(stpc - stp) < fabs(stpq - stp)) ? stpc : stpq;
            if (stp > stx) stpf = fmin(stp + 0.66 * (sty - stp), stpf);
            else stpf = fmax(stp + 0.66 * (sty - stp), stpf);
        } else {
            stpf = (fabs(stpc - stp) > fabs(stpq - stp)) ? stpc : stpq;
            stpf = fmin(stpmax, stpf);
            stpf = fmax(stpmin, stpf);
        }
    } else {
        if (brackt) {
            const double theta = 3 * (fp - fy) / (sty - stp) + dy + dp;
            const double s = fmax(fabs(theta), fmax(fabs(dy), fabs(dp)));
            double gamma = s * sqrt((theta / s) * (theta / s) - (dy / s) * (dp / s));
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

// One call per function value: returns 0 to ask for f, g at the new stp, 1 converged, 2 warning.
__device__ inline int search_step(Search& S, bool start, double f, double g, double& stp, double stpmax) {
    const double ftol = 1e-3, gtol = 0.9, xtol = 0.1, stpmin = 0.0, xtrapl = 1.1, xtrapu = 4.0;
    if (start) {
        S.brackt = false;
        S.stage = 1;
        S.finit = f;
        S.ginit = g;
        S.gtest = ftol * S.ginit;
        S.width = stpmax - stpmin;
        S.width1 = S.width / 0.5;
        S.stx = 0; S.fx = S.finit; S.gx = S.ginit;
        S.sty = 0; S.fy = S.finit; S.gy = S.ginit;
        S.stmin = 0;
        S.stmax = stp + xtrapu * stp;
        return 0;
    }
    const double ftest = S.finit + stp * S.gtest;
    if (S.stage == 1 && f <= ftest && g >= 0) S.stage = 2;
    int task = 0;
    if (S.brackt && (stp <= S.stmin || stp >= S.stmax)) task = 2;
    if (S.brackt && S.stmax - S.stmin <= xtol * S.stmax) task = 2;
    if (stp == stpmax && f <= ftest && g <= S.gtest) task = 2;
    if (stp == stpmin && (f > ftest || g >= S.gtest)) task = 2;
    if (f <= ftest && fabs(g) <= gtol * (-S.ginit)) task = 1;
    if (task) return task;
    if (S.stage == 1 && f <= S.fx && f > ftest) {
        double fm = f - stp * S.gtest, fxm = S.fx - S.stx * S.gtest, fym = S.fy - S.sty * S.gtest;
        double gm = g - S.gtest, gxm = S.gx - S.gtest, gym = S.gy - S.gtest;
        cstep(S.stx, fxm, gxm, S.sty, fym, gym, stp, fm, gm, S.brackt, S.stmin, S.stmax);
        S.fx = fxm + S.stx * S.gtest;
        S.fy = fym + S.sty * S.gtest;
        S.gx = gxm + S.gtest;
        S.gy = gym + S.gtest;
    } else {
        cstep(S.stx, S.fx, S.gx, S.sty, S.fy, S.gy, stp, f, g, S.brackt, S.stmin, S.stmax);
    }
    if (S.brackt) {
        if (fabs(S.sty - S.stx) >= 0.66 * S.width1) stp = S.stx + 0.5 * (S.sty - S.stx);
        S.width1 = S.width;
        S.width = fabs(S.sty - S.stx);
        S.stmin = fmin(S.stx, S.sty);
        S.stmax = fmax(S.stx, S.sty);
    } else {
        S.stmin = stp + xtrapl * (stp - S.stx);
        S.stmax = stp + xtrapu * (stp - S.stx);
    }
    stp = fmax(stp, stpmin);
    stp = fmin(stp, stpmax);
    if ((S.brackt && (stp <= S.stmin || stp >= S.stmax)) || (S.brackt && S.stmax - S.stmin <= xtol * S.stmax))
        stp = S.stx;
    return 0;
}

// L-BFGS-B over n variables, each either free (bounded = false) or with lower bound 0.
struct Lbfgsb {
    QbDiisWork& w;
    int n;
    bool bounded;
    int col, head, tail, iupdat;
    double theta;
    bool updated;

    __device__ Lbfgsb(QbDiisWork& w_, int n_, bool b) : w(w_), n(n_), bounded(b) { refresh(); }

    __device__ void refresh() {
        col = 0;
        head = 0;
        tail = 0;
        iupdat = 0;
        theta = 1.0;
        updated = false;
    }
    __device__ int slot(int k) const { return (head + k) % QB_DS_M; }
    __device__ double& WS(int i, int k) { return w.ws[i + QB_DS_N * slot(k)]; }
    __device__ double& WY(int i, int k) { return w.wy[i + QB_DS_N * slot(k)]; }
    __device__ double& SY(int i, int j) { return w.sy[i + QB_DS_M * j]; }
    __device__ double& SS(int i, int j) { return w.ss[i + QB_DS_M * j]; }

    __device__ double pg_norm(const double* x, const double* g) const {
        double s = 0.0;
        for (int i = 0; i < n; ++i) {
            double gi = g[i];
            if (bounded && gi >= 0) gi = fmin(x[i], gi);   // lower bound 0
            s = fmax(s, fabs(gi));
        }
        return s;
    }

    // p = M v (compact representation's middle matrix), v and p of length 2 col.
    __device__ int middle(const double* v, double* p) {
        if (col == 0) return 0;
        p[col] = v[col];
        for (int i = 1; i < col; ++i) {
            double sum = 0.0;
            for (int k = 0; k < i; ++k) sum += SY(i, k) * v[k] / SY(k, k);
            p[col + i] = v[col + i] + sum;
        }
        if (tri_solve(w.wt, QB_DS_M, col, p + col, true)) return -1;
        for (int i = 0; i < col; ++i) p[i] = v[i] / sqrt(SY(i, i));
        if (tri_solve(w.wt, QB_DS_M, col, p + col, false)) return -1;
        for (int i = 0; i < col; ++i) p[i] = -p[i] / sqrt(SY(i, i));
        for (int i = 0; i < col; ++i) {
            double sum = 0.0;
            for (int k = i + 1; k < col; ++k) sum += SY(k, i) * p[col + k] / SY(i, i);
            p[i] += sum;
        }
        return 0;
    }

    __device__ static void heap_pop(int cnt, double* t, int* ord, bool build) {
        if (build) {
            for (int k = 1; k < cnt; ++k) {
                const double val = t[k];
                const int idx = ord[k];
                int i = k;
                while (i > 0) {
                    const int j = (i + 1) / 2 - 1;
                    if (!(val < t[j])) break;
                    t[i] = t[j];
                    ord[i] = ord[j];
                    i = j;
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
            int i = 0;
            while (true) {
                int j = 2 * (i + 1) - 1;
                if (j > cnt - 2) break;
                if (t[j + 1] < t[j]) j = j + 1;
                if (!(t[j] < val)) break;
                t[i] = t[j];
                ord[i] = ord[j];
                i = j;
            }
            t[i] = val;
            ord[i] = idx;
            t[cnt - 1] = out;
            ord[cnt - 1] = oidx;
        }
    }

    // Generalised Cauchy point: z and c = W^T (z - x); updates where[].
    __device__ int cauchy(const double* x, const double* g, double* xcp, double* c) {
        const int col2 = 2 * col;
        for (int i = 0; i < n; ++i) xcp[i] = x[i];
        if (pg_norm(x, g) <= 0.0) return 0;
        bool bnded = true;
        int nfree = n, nbreak = 0, ibkmin = 0;
        double bkmin = 0.0, f1 = 0.0, tl = 0.0;
        double* p = w.p;
        double* v = w.vv;
        double* wbp = w.wbp;
        double* d = w.d;
        for (int j = 0; j < col2; ++j) p[j] = 0.0;
        for (int i = 0; i < n; ++i) {
            const double neggi = -g[i];
            if (w.where[i] != -1) {   // bounded variable (lower bound 0)
                tl = x[i];
                w.where[i] = 0;
                if (tl <= 0) {
                    if (neggi <= 0) w.where[i] = 1;
                } else if (fabs(neggi) <= 0) {
                    w.where[i] = -3;
                }
            }
            if (w.where[i] != 0 && w.where[i] != -1) {
                d[i] = 0.0;
            } else {
                d[i] = neggi;
                f1 -= neggi * neggi;
                for (int j = 0; j < col; ++j) {
                    p[j] += WY(i, j) * neggi;
                    p[col + j] += WS(i, j) * neggi;
                }
                if (bounded && neggi < 0) {
                    w.ord[nbreak] = i;
                    w.tb[nbreak] = tl / (-neggi);
                    if (nbreak == 0 || w.tb[nbreak] < bkmin) { bkmin = w.tb[nbreak]; ibkmin = nbreak; }
                    ++nbreak;
                } else {
                    --nfree;
                    w.ord[nfree] = i;
                    if (fabs(neggi) > 0) bnded = false;
                }
            }
        }
        if (theta != 1.0)
            for (int j = 0; j < col; ++j) p[col + j] *= theta;
        if (nbreak == 0 && nfree == n) return 0;
        for (int j = 0; j < 2 * QB_DS_M; ++j) c[j] = 0.0;
        double f2 = -theta * f1;
        const double f2_org = f2;
        if (col > 0) {
            if (middle(p, v)) return -1;
            double pv = 0.0;
            for (int j = 0; j < col2; ++j) pv += v[j] * p[j];
            f2 -= pv;
        }
        double dtm = -f1 / f2, tsum = 0.0;
        if (nbreak > 0) {
            int nleft = nbreak, it = 1;
            double tj = 0.0;
            for (int guard = 0; guard <= QB_DS_N; ++guard) {
                const double tj0 = tj;
                int ibp;
                if (it == 1) {
                    tj = bkmin;
                    ibp = w.ord[ibkmin];
                } else {
                    if (it == 2 && ibkmin != nbreak - 1) {
                        w.tb[ibkmin] = w.tb[nbreak - 1];
                        w.ord[ibkmin] = w.ord[nbreak - 1];
                    }
                    heap_pop(nleft, w.tb, w.ord, it == 2);
                    tj = w.tb[nleft - 1];
                    ibp = w.ord[nleft - 1];
                }
                const double dt = tj - tj0;
                if (dtm < dt) break;
                tsum += dt;
                --nleft;
                ++it;
                const double dibp = d[ibp];
                d[ibp] = 0.0;
                const double zibp = -x[ibp];   // to the lower bound 0
                xcp[ibp] = 0.0;
                w.where[ibp] = 1;
                if (nleft == 0 && nbreak == n) {   // every variable fixed
                    if (col > 0)
                        for (int j = 0; j < col2; ++j) c[j] += dt * p[j];
                    return 0;
                }
                const double dibp2 = dibp * dibp;
                f1 = f1 + dt * f2 + dibp2 - theta * dibp * zibp;
                f2 = f2 - theta * dibp2;
                if (col > 0) {
                    for (int j = 0; j < col2; ++j) c[j] += dt * p[j];
                    for (int j = 0; j < col; ++j) {
                        wbp[j] = WY(ibp, j);
                        wbp[col + j] = theta * WS(ibp, j);
                    }
                    if (middle(wbp, v)) return -1;
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
                f2 = fmax(kEps * f2_org, f2);
                if (nleft > 0) {
                    dtm = -f1 / f2;
                } else {
                    if (bnded) {
                        f1 = 0;
                        f2 = 0;
                        dtm = 0;
                    } else {
                        dtm = -f1 / f2;
                    }
                    break;
                }
            }
        }
        if (dtm <= 0) dtm = 0;
        tsum += dtm;
        for (int i = 0; i < n; ++i) xcp[i] += tsum * d[i];
        if (col > 0)
            for (int j = 0; j < col2; ++j) c[j] += dtm * p[j];
        return 0;
    }

    __device__ void collect_free() {
        w.nfree = 0;
        w.nact = 0;
        for (int i = 0; i < n; ++i) {
            if (w.where[i] <= 0) w.freel[w.nfree++] = i;
            else w.actl[w.nact++] = i;
        }
    }

    // LEL^T factor of K = [-D - Y'ZZ'Y/theta, L_a' - R_z'; L_a - R_z, theta S'AA'S] into wn.
    __device__ int form_k() {
        const int ld = 2 * QB_DS_M;
        double* wn = w.wn;
        for (int i = 0; i < ld * ld; ++i) wn[i] = 0.0;
        for (int iy = 0; iy < col; ++iy)
            for (int jy = 0; jy <= iy; ++jy) {
                double yzzy = 0, saas = 0;
                for (int q = 0; q < w.nfree; ++q) {
                    const int k = w.freel[q];
                    yzzy += WY(k, iy) * WY(k, jy);
                }
                for (int q = 0; q < w.nact; ++q) {
                    const int k = w.actl[q];
                    saas += WS(k, iy) * WS(k, jy);
                }
                wn[jy + ld * iy] = yzzy / theta;
                wn[(col + jy) + ld * (col + iy)] = saas * theta;
            }
        for (int iy = 0; iy < col; ++iy) {
            wn[iy + ld * iy] += SY(iy, iy);
            for (int jy = 0; jy < col; ++jy) {
                double val = 0;
                if (jy < iy) {
                    for (int q = 0; q < w.nact; ++q) {
                        const int k = w.actl[q];
                        val += WS(k, iy) * WY(k, jy);
                    }
                    val = -val;
                } else {
                    for (int q = 0; q < w.nfree; ++q) {
                        const int k = w.freel[q];
                        val += WS(k, iy) * WY(k, jy);
                    }
                }
                wn[jy + ld * (col + iy)] = val;
            }
        }
        if (chol_upper(wn, ld, col)) return -1;
        for (int js = col; js < 2 * col; ++js)
            if (tri_solve(wn, ld, col, wn + ld * js, true)) return -1;
        for (int is = col; is < 2 * col; ++is)
            for (int js = is; js < 2 * col; ++js) {
                double s = 0;
                for (int k = 0; k < col; ++k) s += wn[k + ld * is] * wn[k + ld * js];
                wn[is + ld * js] += s;
            }
        if (chol_upper(wn + col + ld * col, ld, col)) return -2;
        return 0;
    }

    __device__ int form_t() {
        for (int j = 0; j < col; ++j) w.wt[QB_DS_M * j] = theta * SS(0, j);
        for (int i = 1; i < col; ++i)
            for (int j = i; j < col; ++j) {
                double s = 0;
                for (int k = 0; k < i; ++k) s += SY(i, k) * SY(j, k) / SY(k, k);
                w.wt[i + QB_DS_M * j] = s + theta * SS(i, j);
            }
        return chol_upper(w.wt, QB_DS_M, col) ? -3 : 0;
    }

    // r = -Z^T (B (z - x) + g) over the free variables.
    __device__ int reduced_gradient(const double* x, const double* g, const double* z, const double* c, double* r) {
        if (!bounded && col > 0) {
            for (int i = 0; i < n; ++i) r[i] = -g[i];
            return 0;
        }
        for (int q = 0; q < w.nfree; ++q) {
            const int k = w.freel[q];
            r[q] = -theta * (z[k] - x[k]) - g[k];
        }
        double* a = w.wv;
        if (middle(c, a)) return -8;
        for (int j = 0; j < col; ++j) {
            const double a1 = a[j], a2 = theta * a[col + j];
            for (int q = 0; q < w.nfree; ++q) {
                const int k = w.freel[q];
                r[q] += WY(k, j) * a1 + WS(k, j) * a2;
            }
        }
        return 0;
    }

    // Subspace Newton step from the Cauchy point z (in place), projection, backtracking.
    __device__ int subspace_min(const double* xx, const double* gg, double* x, double* d) {
        const int ld = 2 * QB_DS_M, nsub = w.nfree;
        double* wv = w.wv;
        for (int i = 0; i < col; ++i) {
            double t1 = 0, t2 = 0;
            for (int j = 0; j < nsub; ++j) {
                const int k = w.freel[j];
                t1 += WY(k, i) * d[j];
                t2 += WS(k, i) * d[j];
            }
            wv[i] = t1;
            wv[col + i] = theta * t2;
        }
        if (tri_solve(w.wn, ld, 2 * col, wv, true)) return -1;
        for (int i = 0; i < col; ++i) wv[i] = -wv[i];
        if (tri_solve(w.wn, ld, 2 * col, wv, false)) return -1;
        for (int jy = 0; jy < col; ++jy)
            for (int i = 0; i < nsub; ++i) {
                const int k = w.freel[i];
                d[i] += WY(k, jy) * wv[jy] / theta + WS(k, jy) * wv[col + jy];
            }
        for (int i = 0; i < nsub; ++i) d[i] /= theta;
        double* xp = w.xp;
        for (int i = 0; i < n; ++i) xp[i] = x[i];
        bool hit = false;
        for (int i = 0; i < nsub; ++i) {
            const int k = w.freel[i];
            if (!bounded) {
                x[k] = x[k] + d[i];
            } else {
                x[k] = fmax(0.0, x[k] + d[i]);
                if (x[k] == 0.0) hit = true;
            }
        }
        if (!hit) return 0;
        double ddp = 0;
        for (int i = 0; i < n; ++i) ddp += (x[i] - xx[i]) * gg[i];
        if (ddp <= 0) return 0;
        for (int i = 0; i < n; ++i) x[i] = xp[i];
        double alpha = 1.0, temp1 = alpha;
        int ibd = -1;
        for (int i = 0; i < nsub; ++i) {
            const int k = w.freel[i];
            const double dk = d[i];
            if (!bounded) continue;
            if (dk < 0) {
                const double t2 = -x[k];
                if (t2 >= 0) temp1 = 0;
                else if (dk * alpha < t2) temp1 = t2 / dk;
            }
            if (temp1 < alpha) {
                alpha = temp1;
                ibd = i;
            }
        }
        if (alpha < 1.0 && ibd >= 0 && d[ibd] < 0) {
            x[w.freel[ibd]] = 0.0;
            d[ibd] = 0;
        }
        for (int i = 0; i < nsub; ++i) x[w.freel[i]] += alpha * d[i];
        return 0;
    }

    __device__ void update_memory(const double* s, const double* y, double rr, double dr, double stp, double dtd) {
        if (iupdat <= QB_DS_M) {
            col = iupdat;
            tail = (head + iupdat - 1) % QB_DS_M;
        } else {
            tail = (tail + 1) % QB_DS_M;
            head = (head + 1) % QB_DS_M;
        }
        for (int i = 0; i < n; ++i) {
            w.ws[i + QB_DS_N * tail] = s[i];
            w.wy[i + QB_DS_N * tail] = y[i];
        }
        theta = rr / dr;
        if (iupdat > QB_DS_M) {
            for (int j = 0; j < col - 1; ++j) {
                for (int i = 0; i <= j; ++i) SS(i, j) = SS(i + 1, j + 1);
                for (int i = j; i < col - 1; ++i) SY(i, j) = SY(i + 1, j + 1);
            }
        }
        for (int j = 0; j < col - 1; ++j) {
            double a = 0, b = 0;
            for (int i = 0; i < n; ++i) {
                a += s[i] * WY(i, j);
                b += WS(i, j) * s[i];
            }
            SY(col - 1, j) = a;
            SS(j, col - 1) = b;
        }
        SS(col - 1, col - 1) = (stp == 1.0) ? dtd : stp * stp * dtd;
        SY(col - 1, col - 1) = dr;
    }

    // Minimise from w.x (in place); factr 1e5, pgtol 1e-15, 10000 iterations / evaluations.
    __device__ int run() {
        const double tol = 1e5 * kEps, pgtol = 1e-15;
        const int maxiter = 10000, maxfun = 10000;
        double *x = w.x, *g = w.g, *z = w.z, *d = w.d, *r = w.r, *xs = w.xs, *gs = w.gs;
        for (int i = 0; i < n; ++i) {
            if (bounded && x[i] < 0.0) x[i] = 0.0;
            w.where[i] = bounded ? 0 : -1;
        }
        w.nfree = 0;
        w.nact = 0;
        double f = fg(w, n, x, g);
        int nfgv = 1, iter = 0;
        if (pg_norm(x, g) <= pgtol) return iter;
        for (int outer = 0; outer < 4 * maxiter; ++outer) {
            if (!bounded && col > 0) {
                for (int i = 0; i < n; ++i) z[i] = x[i];
            } else {
                if (cauchy(x, g, z, w.cw) != 0) { refresh(); continue; }
                collect_free();
            }
            if (w.nfree > 0 && col > 0) {
                if (form_k() != 0) { refresh(); continue; }
                if (reduced_gradient(x, g, z, w.cw, r) != 0) { refresh(); continue; }
                if (subspace_min(x, g, z, r) != 0) { refresh(); continue; }
            }
            for (int i = 0; i < n; ++i) d[i] = z[i] - x[i];
            double dtd = 0.0;
            for (int i = 0; i < n; ++i) dtd += d[i] * d[i];
            const double dnorm = sqrt(dtd);
            double stpmx = 1e10;
            if (bounded) {
                if (iter == 0) {
                    stpmx = 1.0;
                } else {
                    for (int i = 0; i < n; ++i) {
                        const double a1 = d[i];
                        if (a1 < 0) {
                            const double a2 = -x[i];
                            if (a2 >= 0) stpmx = 0;
                            else if (a1 * stpmx < a2) stpmx = a2 / a1;
                        }
                    }
                }
            }
            double stp = (iter == 0) ? fmin(1.0 / dnorm, stpmx) : 1.0;
            for (int i = 0; i < n; ++i) {
                xs[i] = x[i];
                gs[i] = g[i];
            }
            const double fold = f;
            int ifun = 0, iback = 0;
            double gd = 0, gdold = 0;
            Search S;
            bool newx = false, start = true;
            for (int ls = 0; ls < 64; ++ls) {
                gd = 0.0;
                for (int i = 0; i < n; ++i) gd += g[i] * d[i];
                if (ifun == 0) {
                    gdold = gd;
                    if (gd >= 0) break;   // not a descent direction
                }
                const int st = search_step(S, start, f, gd, stp, stpmx);
                start = false;
                if (st == 0) {
                    ++ifun;
                    ++nfgv;
                    iback = ifun - 1;
                    if (stp == 1.0) {
                        for (int i = 0; i < n; ++i) x[i] = z[i];
                    } else {
                        for (int i = 0; i < n; ++i) x[i] = stp * d[i] + xs[i];
                    }
                    if (iback >= 20) break;
                    f = fg(w, n, x, g);
                    continue;
                }
                newx = true;
                break;
            }
            if (!newx) {
                for (int i = 0; i < n; ++i) {
                    x[i] = xs[i];
                    g[i] = gs[i];
                }
                f = fold;
                if (col == 0) return iter + 1;
                refresh();
                continue;
            }
            ++iter;
            const double sbgnrm = pg_norm(x, g);
            if (iter >= maxiter || nfgv >= maxfun) return iter;
            if (sbgnrm <= pgtol) return iter;
            const double ddum0 = fmax(fmax(fabs(fold), fabs(f)), 1.0);
            if (fold - f <= tol * ddum0) return iter;
            double rr = 0.0;
            for (int i = 0; i < n; ++i) {
                r[i] = g[i] - gs[i];
                rr += r[i] * r[i];
            }
            double dr, ddum;
            if (stp == 1.0) {
                dr = gd - gdold;
                ddum = -gdold;
            } else {
                dr = (gd - gdold) * stp;
                for (int i = 0; i < n; ++i) d[i] *= stp;
                ddum = -gdold * stp;
            }
            if (dr <= kEps * ddum) {
                updated = false;
                continue;
            }
            updated = true;
            ++iupdat;
            update_memory(d, r, rr, dr, stp, dtd);
            if (form_t() != 0) { refresh(); continue; }
        }
        return iter;
    }
};

// SPG2 with lower bound 0 (bounded) or none.
__device__ inline int spg(QbDiisWork& w, int n, bool bounded) {
    const double lmin = 1e-30, lmax = 1e30, gamma = 1e-4, sigma1 = 0.1, sigma2 = 0.9, eps = 1e-15;
    const int nitmax = 10000, nfevalmax = 10000, mem = 20;
    double *x = w.x, *g = w.g, *xn = w.z, *gn = w.r, *dv = w.d;
    auto pg_norm = [&](const double* xv, const double* gv) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) {
            double t = xv[i] - gv[i];
            if (bounded) t = fmax(t, 0.0);
            s = fmax(s, fabs(t - xv[i]));
        }
        return s;
    };
    if (bounded)
        for (int i = 0; i < n; ++i) x[i] = fmax(x[i], 0.0);
    double fc = obj_f(w, n, x);
    obj_g(w, n, x, g);
    int nfeval = 1, nit = 0;
    double gnorm = pg_norm(x, g);
    if (gnorm <= eps) return 0;
    for (int i = 0; i < mem; ++i) w.fprev[i] = fc;
    double lam = fmin(lmax, fmax(lmin, 1.0 / gnorm));
    while (nit < nitmax) {
        for (int i = 0; i < n; ++i) {
            double t = x[i] - lam * g[i];
            if (bounded) t = fmax(t, 0.0);
            dv[i] = t - x[i];
        }
        double gtd = 0.0, fref = w.fprev[0];
        for (int i = 0; i < n; ++i) gtd += g[i] * dv[i];
        for (int i = 1; i < mem; ++i) fref = fmax(fref, w.fprev[i]);
        double alpha = 1.0;
        for (int i = 0; i < n; ++i) xn[i] = x[i] + alpha * dv[i];
        double fn = obj_f(w, n, xn);
        ++nfeval;
        while (fn > fref + gamma * alpha * gtd) {
            const double atemp = -0.5 * gtd * alpha * alpha / (fn - fc - alpha * gtd);
            if (atemp >= sigma1 && atemp <= sigma2 * alpha) alpha = atemp;
            else alpha /= 2;
            for (int i = 0; i < n; ++i) xn[i] = x[i] + alpha * dv[i];
            fn = obj_f(w, n, xn);
            if (++nfeval > nfevalmax) {
                for (int i = 0; i < n; ++i) x[i] = xn[i];
                return 2;
            }
        }
        ++nit;
        w.fprev[nit % mem] = fn;
        obj_g(w, n, xn, gn);
        double sts = 0, sty = 0;
        for (int i = 0; i < n; ++i) {
            const double s = xn[i] - x[i], y = gn[i] - g[i];
            sts += s * s;
            sty += s * y;
        }
        lam = sty <= 0 ? lmax : fmin(lmax, fmax(lmin, sts / sty));
        for (int i = 0; i < n; ++i) {
            x[i] = xn[i];
            g[i] = gn[i];
        }
        fc = fn;
        gnorm = pg_norm(x, g);
        if (gnorm <= eps) return 0;
    }
    return 1;
}

// LU with partial pivoting of the leading n x n block of A (column-major, leading dimension
// n), solving A x = b in place of b; returns the determinant (0 when a pivot vanishes).
__device__ inline double lu_solve(int n, double* A, double* b) {
    double det = 1.0;
    for (int k = 0; k < n; ++k) {
        int p = k;
        for (int i = k + 1; i < n; ++i)
            if (fabs(A[i + n * k]) > fabs(A[p + n * k])) p = i;
        if (A[p + n * k] == 0.0) return 0.0;
        if (p != k) {
            for (int j = 0; j < n; ++j) {
                const double t = A[k + n * j];
                A[k + n * j] = A[p + n * j];
                A[p + n * j] = t;
            }
            const double t = b[k];
            b[k] = b[p];
            b[p] = t;
            det = -det;
        }
        const double pv = A[k + n * k];
        det *= pv;
        for (int i = k + 1; i < n; ++i) {
            const double f = A[i + n * k] / pv;
            A[i + n * k] = f;
            for (int j = k + 1; j < n; ++j) A[i + n * j] -= f * A[k + n * j];
            b[i] -= f * b[k];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        double t = b[i];
        for (int j = i + 1; j < n; ++j) t -= A[i + n * j] * b[j];
        b[i] = t / A[i + n * i];
    }
    return det;
}

}  // namespace qbds

// CMsolver! (HartreeFock.jl:1445-1477) by one thread: solve [B 1; 1 0][c; l] = [-v; 1]; if
// `convex` and some c < 0, try the subsystems with index subsets removed (by increasing
// size, smallest |c| first) until a non-negative solution appears; a singular bordered
// matrix gets B += 4e-13 I (1000 getAtolVal).  B is m x m with leading dimension ldb, m <= 16.
// Bounded: at most 64 perturbation rounds; returns false if they run out (c then holds the
// last candidate).
static __device__ __noinline__ bool qb_cm_solve(QbDiisWork& w, int m, int convex, const double* Bin, int ldb,
                                                const double* v, double* c) {
    const int M = m + 1;
    double *B = w.cmB, *A = w.cmA, *W = w.cmW, *b = w.cmb, *x = w.cmx;
    for (int j = 0; j < m; ++j)
        for (int i = 0; i < m; ++i) B[i + m * j] = Bin[i + ldb * j];
    for (int round = 0; round < 64; ++round) {
        for (int guard = 0; guard < 64; ++guard) {
            for (int j = 0; j < M; ++j)
                for (int i = 0; i < M; ++i)
                    A[i + M * j] = (i < m && j < m) ? B[i + m * j] : ((i == m && j == m) ? 0.0 : 1.0);
            for (int i = 0; i < M * M; ++i) W[i] = A[i];
            for (int i = 0; i < M; ++i) x[i] = 0.0;
            if (qbds::lu_solve(M, W, x) != 0.0) break;
            for (int i = 0; i < m; ++i) B[i + m * i] += 4e-13;
        }
        for (int i = 0; i < m; ++i) b[i] = v ? -v[i] : 0.0;
        b[m] = 1.0;
        for (int i = 0; i < M * M; ++i) W[i] = A[i];
        for (int i = 0; i < M; ++i) x[i] = b[i];
        qbds::lu_solve(M, W, x);
        bool neg = false;
        for (int i = 0; i < m; ++i) {
            c[i] = x[i];
            neg |= x[i] < 0.0;
        }
        if (!convex || !neg) return true;
        int perm[QB_DS_N];
        for (int i = 0; i < m; ++i) perm[i] = i;
        for (int i = 1; i < m; ++i) {   // stable insertion sort by |c|
            const int t = perm[i];
            int j = i - 1;
            while (j >= 0 && fabs(c[perm[j]]) > fabs(c[t])) {
                perm[j + 1] = perm[j];
                --j;
            }
            perm[j + 1] = t;
        }
        for (int sz = 1; sz <= m; ++sz) {
            int comb[QB_DS_N];
            for (int t = 0; t < sz; ++t) comb[t] = t;
            while (true) {
                unsigned drop = 0;
                for (int t = 0; t < sz; ++t) drop |= 1u << perm[comb[t]];
                int keep[QB_DS_N + 1], k = 0;
                for (int i = 0; i <= m; ++i)
                    if (!(drop >> i & 1u)) keep[k++] = i;
                for (int jj = 0; jj < k; ++jj) {
                    x[jj] = b[keep[jj]];
                    for (int ii = 0; ii < k; ++ii) W[ii + k * jj] = A[keep[ii] + M * keep[jj]];
                }
                if (qbds::lu_solve(k, W, x) != 0.0) {
                    bool bad = false;
                    for (int i = 0; i < m; ++i) c[i] = 0.0;
                    for (int jj = 0; jj < k - 1; ++jj) c[keep[jj]] = x[jj];
                    for (int i = 0; i < m; ++i) bad |= c[i] < 0.0;
                    if (!bad) return true;
                }
                int pos = sz - 1;
                while (pos >= 0 && comb[pos] == m - sz + pos) --pos;
                if (pos < 0) break;
                ++comb[pos];
                for (int t = pos + 1; t < sz; ++t) comb[t] = comb[t - 1] + 1;
            }
        }
        for (int i = 0; i < m; ++i) B[i + m * i] += 4e-13;
    }
    return false;
}

// One thread: solve the DIIS coefficient problem of m entries.  B (m x m, leading
// dimension ldb) and v (m) describe it; c (m) is the starting point on entry and the
// normalised coefficients on return.  solver: QB_DIIS_LBFGS or QB_DIIS_SPGB; convex adds
// c >= 0.  Returns the solver's iteration count (L-BFGS-B) or status (SPG).
static __device__ __noinline__ int qb_diis_iterative_solve(QbDiisWork& w, int solver, int convex, int m, const double* B,
                                                    int ldb, const double* v, double* c) {
    for (int j = 0; j < m; ++j) {
        w.v[j] = v ? v[j] : 0.0;
        for (int i = 0; i < m; ++i) w.B[i + QB_DS_N * j] = B[i + ldb * j];
        w.x[j] = c[j];
    }
    int out;
    if (solver == QB_DIIS_SPGB) {
        out = qbds::spg(w, m, convex != 0);
    } else {
        qbds::Lbfgsb opt(w, m, convex != 0);
        out = opt.run();
    }
    w.iters = out;
    const double s = qbds::shifted_sum(m, w.x);
    for (int i = 0; i < m; ++i) c[i] = w.x[i] / s;
    return out;
}
