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
// One warp runs a solve.  The problems have at most 16 variables and 15 correction pairs
// (30 rows in the compact L-BFGS-B matrices), so lane i owns variable i, or row / column i
// of a small matrix, and the scalar control (line search, breakpoint walk, stopping tests)
// runs alike in every lane from values that every lane holds.  GB300 issues an FP64 warp
// instruction in about 64 cycles per SM sub-partition whether one lane or 32 are active, so
// a one-thread solver pays that for every scalar operation; spreading the vector and matrix
// loops over the lanes divides the instruction count by up to 32.  Sums over lanes are
// butterfly reductions, which give the same value in every lane.  The state lives in a
// QbDiisWork block in shared memory supplied by the caller (about 27 KB).  Every loop is
// bounded (10000 iterations and evaluations, 20 trial steps per line search, as in the
// reference's settings).  The starting point is c on entry (the previous solution with a 1
// appended for the newest entry, as the reference's per-method coefficient vector carries
// over); on return c holds the normalised solution.  All 32 lanes of the warp must call the
// entry points together.
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
    double rinv[2 * QB_DS_M];            // reciprocal diagonal of a triangular factor
    double dinv[QB_DS_M], sqinv[QB_DS_M];  // 1 / SY(k,k) and 1 / sqrt(SY(k,k))
    double fprev[20];
    double cmB[QB_DS_N * QB_DS_N], cmA[(QB_DS_N + 1) * (QB_DS_N + 1)], cmW[(QB_DS_N + 1) * (QB_DS_N + 1)];
    double cmb[QB_DS_N + 1], cmx[QB_DS_N + 1];
    int where[QB_DS_N], freel[QB_DS_N];
    int iters;   // solver iterations of the last solve (diagnostics)
};

namespace qbds {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kEps = 2.220446049250313e-16;
constexpr double kShift = 4e-16;   // getAtolVal(Float64) (src/Arithmetic.jl:42)

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

__device__ __forceinline__ double wsum(double a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
    return a;
}

__device__ __forceinline__ double wmax(double a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = fmax(a, __shfl_xor_sync(kFull, a, o));
    return a;
}

// Smallest value over the lanes and the lowest lane holding it.
__device__ __forceinline__ double wargmin(double a, int& at) {
    double m = a;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(kFull, m, o));
    at = __ffs(__ballot_sync(kFull, a == m)) - 1;
    return m;
}

__device__ __forceinline__ bool wany(bool p) { return __any_sync(kFull, p); }

// shiftLastEle! on the iterate
__device__ inline double shifted_sum(int n, double* c) {
    const int l = lane_id();
    double s = wsum(l < n ? c[l] : 0.0);
    if (s < kShift) {
        const double sh = (s < 0 ? -1.0 : 1.0) * kShift;
        s += sh;
        __syncwarp();
        if (l == n - 1) c[l] += sh;
        __syncwarp();
    }
    return s;
}

// v.c and c^T B c
__device__ inline void parts(const QbDiisWork& w, int n, const double* c, double& vc, double& cBc) {
    const int l = lane_id();
    double t = 0.0, cl = 0.0, vl = 0.0;
    if (l < n) {
        cl = c[l];
        vl = w.v[l];
        for (int i = 0; i < n; ++i) t = fma(c[i], w.B[i + QB_DS_N * l], t);
    }
    vc = wsum(vl * cl);
    cBc = wsum(t * cl);
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
    const int l = lane_id();
    if (l < n) {
        double bc = 0.0;
        for (int j = 0; j < n; ++j) bc = fma(w.B[l + QB_DS_N * j] + w.B[j + QB_DS_N * l], c[j], bc);
        g[l] = w.v[l] / s + bc / (2 * s * s) - common;
    }
    __syncwarp();
}

__device__ inline double fg(const QbDiisWork& w, int n, double* c, double* g) {
    const double f = obj_f(w, n, c);
    obj_g(w, n, c, g);
    return f;
}

// Cholesky R^T R of the leading k x k block (k <= 32), upper R in place, right-looking:
// lane l owns column l.  Nonzero (the failing column + 1) on a non-positive pivot.
__device__ inline int chol_upper(double* a, int ld, int k) {
    const int l = lane_id();
    __syncwarp();
    for (int j = 0; j < k; ++j) {
        const double djj = a[j + ld * j];
        if (djj <= 0.0) return j + 1;
        const double rj = sqrt(djj), ri = 1.0 / rj;
        const bool mine = l > j && l < k;
        double ajl = 0.0;
        if (mine) ajl = a[j + ld * l] * ri;
        __syncwarp();
        if (mine) a[j + ld * l] = ajl;
        if (l == j) a[j + ld * j] = rj;
        __syncwarp();
        if (mine)
            for (int i = j + 1; i <= l; ++i) a[i + ld * l] = fma(-a[j + ld * i], ajl, a[i + ld * l]);
        __syncwarp();
    }
    return 0;
}

// R^T x = b (trans) or R x = b, R upper k x k (k <= 32), in place of b; lane l owns b_l.
// Nonzero (the first zero pivot + 1) on a zero pivot.
__device__ inline int tri_solve(const double* r, int ld, int k, double* b, bool trans) {
    const int l = lane_id();
    __syncwarp();
    const double dl = l < k ? r[l + ld * l] : 1.0;
    const unsigned zero = __ballot_sync(kFull, l < k && dl == 0.0);
    if (zero) return __ffs(zero);
    const double rl = 1.0 / dl;
    double bl = l < k ? b[l] : 0.0;
    if (trans) {
        for (int i = 0; i < k; ++i) {
            if (l == i) bl *= rl;
            const double bi = __shfl_sync(kFull, bl, i);
            if (l > i && l < k) bl = fma(-r[i + ld * l], bi, bl);
        }
    } else {
        for (int i = k - 1; i >= 0; --i) {
            if (l == i) bl *= rl;
            const double bi = __shfl_sync(kFull, bl, i);
            if (l < i) bl = fma(-r[l + ld * i], bi, bl);
        }
    }
    __syncwarp();
    if (l < k) b[l] = bl;
    __syncwarp();
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
// The correction pairs sit in the columns of ws / wy in a ring (slot(k) = (head + k) mod m).
struct Lbfgsb {
    QbDiisWork& w;
    int n;
    bool bounded;
    int col, head, tail, iupdat, nfree;
    double theta;

    __device__ Lbfgsb(QbDiisWork& w_, int n_, bool b) : w(w_), n(n_), bounded(b), nfree(0) { refresh(); }

    __device__ void refresh() {
        col = 0;
        head = 0;
        tail = 0;
        iupdat = 0;
        theta = 1.0;
    }
    __device__ int slot(int k) const { return (head + k) % QB_DS_M; }
    __device__ const double* ycol(int k) const { return w.wy + QB_DS_N * slot(k); }
    __device__ const double* scol(int k) const { return w.ws + QB_DS_N * slot(k); }
    __device__ double& SY(int i, int j) { return w.sy[i + QB_DS_M * j]; }
    __device__ double& SS(int i, int j) { return w.ss[i + QB_DS_M * j]; }

    // infinity norm of the projected gradient
    __device__ double pg_norm(const double* x, const double* g) const {
        const int l = lane_id();
        double gi = 0.0;
        if (l < n) {
            gi = g[l];
            if (bounded && gi >= 0) gi = fmin(x[l], gi);   // lower bound 0
        }
        return wmax(fabs(gi));
    }

    // p = M v (compact representation's middle matrix), v and p of length 2 col.
    __device__ int middle(const double* v, double* p) {
        if (col == 0) return 0;
        const int l = lane_id();
        __syncwarp();
        if (l < col) {
            double sum = 0.0;
            for (int k = 0; k < l; ++k) sum = fma(SY(l, k) * v[k], w.dinv[k], sum);
            p[col + l] = v[col + l] + sum;
        }
        if (tri_solve(w.wt, QB_DS_M, col, p + col, true)) return -1;
        if (l < col) p[l] = v[l] * w.sqinv[l];
        if (tri_solve(w.wt, QB_DS_M, col, p + col, false)) return -1;
        if (l < col) p[l] = -p[l] * w.sqinv[l];
        __syncwarp();
        if (l < col) {
            double sum = 0.0;
            for (int k = l + 1; k < col; ++k) sum = fma(SY(k, l), p[col + k], sum);
            p[l] += sum * w.dinv[l];
        }
        __syncwarp();
        return 0;
    }

    // Generalised Cauchy point xcp and c = W^T (xcp - x); updates where[].  The breakpoints
    // are visited in increasing order by a warp minimum over the lanes still to be visited
    // (equal breakpoints in increasing variable order).
    __device__ int cauchy(const double* x, const double* g, double* xcp, double* c) {
        const int l = lane_id(), col2 = 2 * col;
        const bool own = l < n;
        const double xl = own ? x[l] : 0.0, gl = own ? g[l] : 0.0;
        if (own) xcp[l] = xl;
        __syncwarp();
        if (pg_norm(x, g) <= 0.0) return 0;
        const double neggi = -gl;
        int wh = own ? w.where[l] : -2;
        if (own && wh != -1) {   // bounded variable (lower bound 0)
            wh = 0;
            if (xl <= 0) {
                if (neggi <= 0) wh = 1;
            } else if (fabs(neggi) <= 0) {
                wh = -3;
            }
        }
        const bool moving = own && (wh == 0 || wh == -1);
        double dl = moving ? neggi : 0.0;
        double f1 = -wsum(moving ? neggi * neggi : 0.0);
        const bool brk = moving && bounded && neggi < 0;
        const bool fre = moving && !brk;
        double my_tb = brk ? xl / (-neggi) : INFINITY;
        const int nbreak = __popc(__ballot_sync(kFull, brk));
        const int nfree0 = n - __popc(__ballot_sync(kFull, fre));
        const bool bnded = !wany(fre && fabs(neggi) > 0);
        if (own) {
            w.d[l] = dl;
            w.where[l] = wh;
        }
        __syncwarp();
        double* p = w.p;
        double* v = w.vv;
        double* wbp = w.wbp;
        if (l < col2) {   // p = W^T d
            const double* src = l < col ? ycol(l) : scol(l - col);
            double s = 0.0;
            for (int i = 0; i < n; ++i) s = fma(src[i], w.d[i], s);
            if (l >= col) s *= theta;
            p[l] = s;
        }
        __syncwarp();
        if (nbreak == 0 && nfree0 == n) return 0;
        if (l < 2 * QB_DS_M) c[l] = 0.0;
        double f2 = -theta * f1;
        const double f2_org = f2;
        if (col > 0) {
            if (middle(p, v)) return -1;
            f2 -= wsum(l < col2 ? v[l] * p[l] : 0.0);
        }
        double dtm = -f1 / f2, tsum = 0.0;
        double cl = 0.0, pl = l < col2 ? p[l] : 0.0;   // lane l owns c[l], p[l]
        if (nbreak > 0) {
            int nleft = nbreak;
            double tj = 0.0;
            for (int guard = 0; guard <= QB_DS_N; ++guard) {
                const double tj0 = tj;
                int ibp;
                tj = wargmin(my_tb, ibp);
                const double dt = tj - tj0;
                if (dtm < dt) break;
                tsum += dt;
                --nleft;
                const double dibp = __shfl_sync(kFull, dl, ibp);
                const double zibp = -__shfl_sync(kFull, xl, ibp);   // to the lower bound 0
                if (l == ibp) {
                    my_tb = INFINITY;
                    dl = 0.0;
                    wh = 1;
                    xcp[l] = 0.0;
                    w.where[l] = 1;
                }
                if (nleft == 0 && nbreak == n) {   // every variable fixed
                    if (col > 0 && l < col2) c[l] = fma(dt, pl, cl);
                    __syncwarp();
                    return 0;
                }
                const double dibp2 = dibp * dibp;
                f1 = f1 + dt * f2 + dibp2 - theta * dibp * zibp;
                f2 = f2 - theta * dibp2;
                if (col > 0) {
                    cl = fma(dt, pl, cl);
                    if (l < col2) {
                        c[l] = cl;
                        wbp[l] = l < col ? ycol(l)[ibp] : theta * scol(l - col)[ibp];
                    }
                    if (middle(wbp, v)) return -1;
                    const double vl = l < col2 ? v[l] : 0.0, wl = l < col2 ? wbp[l] : 0.0;
                    const double wmc = wsum(cl * vl), wmp = wsum(pl * vl), wmw = wsum(wl * vl);
                    pl = fma(-dibp, wl, pl);
                    if (l < col2) p[l] = pl;
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
        __syncwarp();
        if (own) {
            xcp[l] = fma(tsum, dl, xcp[l]);
            w.d[l] = dl;
        }
        if (col > 0 && l < col2) c[l] = fma(dtm, pl, cl);
        __syncwarp();
        return 0;
    }

    // freel = the variables with where <= 0 in increasing order; nfree their count
    __device__ void collect_free() {
        const int l = lane_id();
        const bool fr = l < n && w.where[l] <= 0;
        const unsigned fm = __ballot_sync(kFull, fr);
        if (fr) w.freel[__popc(fm & ((1u << l) - 1u))] = l;
        nfree = __popc(fm);
        __syncwarp();
    }

    // LEL^T factor of K = [-D - Y'ZZ'Y/theta, L_a' - R_z'; L_a - R_z, theta S'AA'S] into wn
    // (Z: free variables, A: active ones).
    __device__ int form_k() {
        const int ld = 2 * QB_DS_M, l = lane_id();
        double* wn = w.wn;
        for (int i = l; i < ld * ld; i += 32) wn[i] = 0.0;
        __syncwarp();
        for (int e = l; e < col * col; e += 32) {
            const int jy = e % col, iy = e / col;
            const double *yi = ycol(iy), *yj = ycol(jy), *si = scol(iy);
            const double* sj = scol(jy);
            const bool upper = jy <= iy, strict = jy < iy;
            double yzzy = 0, saas = 0, cross = 0;
            for (int k = 0; k < n; ++k) {
                const bool fr = w.where[k] <= 0;
                yzzy = fma(fr ? yi[k] : 0.0, yj[k], yzzy);
                saas = fma(fr ? 0.0 : si[k], sj[k], saas);
                cross = fma((strict != fr) ? si[k] : 0.0, yj[k], cross);
            }
            if (upper) {
                wn[jy + ld * iy] = yzzy / theta + (jy == iy ? SY(iy, iy) : 0.0);
                wn[(col + jy) + ld * (col + iy)] = saas * theta;
            }
            wn[jy + ld * (col + iy)] = strict ? -cross : cross;
        }
        if (chol_upper(wn, ld, col)) return -1;
        // columns col .. 2 col - 1 of the top block rows: R^T X = B, one column per lane
        {
            const double dl = l < col ? wn[l + ld * l] : 1.0;
            if (wany(l < col && dl == 0.0)) return -1;
            if (l < col) w.rinv[l] = 1.0 / dl;
            __syncwarp();
            if (l < col) {
                double* bcol = wn + ld * (col + l);
                for (int i = 0; i < col; ++i) {
                    double t = bcol[i];
                    for (int q = 0; q < i; ++q) t = fma(-wn[q + ld * i], bcol[q], t);
                    bcol[i] = t * w.rinv[i];
                }
            }
            __syncwarp();
        }
        for (int e = l; e < col * col; e += 32) {
            const int a = e % col, b = e / col;
            if (a <= b) {
                const double *ca = wn + ld * (col + a), *cb = wn + ld * (col + b);
                double s = 0;
                for (int k = 0; k < col; ++k) s = fma(ca[k], cb[k], s);
                wn[(col + a) + ld * (col + b)] += s;
            }
        }
        if (chol_upper(wn + col + ld * col, ld, col)) return -2;
        return 0;
    }

    // T = theta S'S + L D^-1 L', factored; also the reciprocals of SY's diagonal.
    __device__ int form_t() {
        const int l = lane_id();
        if (l < col) {
            const double dk = SY(l, l);
            w.dinv[l] = 1.0 / dk;
            w.sqinv[l] = 1.0 / sqrt(dk);
        }
        __syncwarp();
        for (int e = l; e < col * col; e += 32) {
            const int i = e % col, j = e / col;
            if (i <= j) {
                double s = 0;
                for (int k = 0; k < i; ++k) s = fma(SY(i, k) * SY(j, k), w.dinv[k], s);
                w.wt[i + QB_DS_M * j] = (i == 0) ? theta * SS(0, j) : s + theta * SS(i, j);
            }
        }
        return chol_upper(w.wt, QB_DS_M, col) ? -3 : 0;
    }

    // r = -Z^T (B (z - x) + g) over the free variables (r indexed by the free list).
    __device__ int reduced_gradient(const double* x, const double* g, const double* z, const double* c, double* r) {
        const int l = lane_id();
        if (!bounded && col > 0) {
            if (l < n) r[l] = -g[l];
            __syncwarp();
            return 0;
        }
        double* a = w.wv;
        if (middle(c, a)) return -8;
        if (l < nfree) {
            const int k = w.freel[l];
            double rq = -theta * (z[k] - x[k]) - g[k];
            for (int j = 0; j < col; ++j) {
                const double a1 = a[j], a2 = theta * a[col + j];
                rq += ycol(j)[k] * a1 + scol(j)[k] * a2;
            }
            r[l] = rq;
        }
        __syncwarp();
        return 0;
    }

    // Subspace Newton step from the Cauchy point x (= z, in place), projection, backtracking;
    // d holds the reduced gradient over the free list on entry.
    __device__ int subspace_min(const double* xx, const double* gg, double* x, double* d) {
        const int ld = 2 * QB_DS_M, nsub = nfree, l = lane_id(), col2 = 2 * col;
        double* wv = w.wv;
        if (l < col2) {
            const double* src = l < col ? ycol(l) : scol(l - col);
            double t = 0;
            for (int j = 0; j < nsub; ++j) t = fma(src[w.freel[j]], d[j], t);
            wv[l] = l < col ? t : theta * t;
        }
        if (tri_solve(w.wn, ld, col2, wv, true)) return -1;
        if (l < col) wv[l] = -wv[l];
        if (tri_solve(w.wn, ld, col2, wv, false)) return -1;
        if (l < col) wv[l] /= theta;
        __syncwarp();
        if (l < nsub) {
            const int k = w.freel[l];
            double dq = d[l];
            for (int jy = 0; jy < col; ++jy) dq += ycol(jy)[k] * wv[jy] + scol(jy)[k] * wv[col + jy];
            d[l] = dq / theta;
        }
        if (l < n) w.xp[l] = x[l];
        __syncwarp();
        bool hitl = false;
        if (l < nsub) {
            const int k = w.freel[l];
            double nx = x[k] + d[l];
            if (bounded) {
                nx = fmax(0.0, nx);
                hitl = nx == 0.0;
            }
            x[k] = nx;
        }
        __syncwarp();
        if (!wany(hitl)) return 0;
        const double ddp = wsum(l < n ? (x[l] - xx[l]) * gg[l] : 0.0);
        if (ddp <= 0) return 0;
        if (l < n) x[l] = w.xp[l];
        __syncwarp();
        // the longest feasible step along d (every lane walks the free list alike)
        double alpha = 1.0, temp1 = alpha;
        int ibd = -1;
        for (int i = 0; i < nsub; ++i) {
            const int k = w.freel[i];
            const double dk = d[i];
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
        const bool pin = alpha < 1.0 && ibd >= 0 && d[ibd] < 0;
        __syncwarp();
        if (pin && l == 0) {
            x[w.freel[ibd]] = 0.0;
            d[ibd] = 0;
        }
        __syncwarp();
        if (l < nsub) x[w.freel[l]] += alpha * d[l];
        __syncwarp();
        return 0;
    }

    __device__ void update_memory(const double* s, const double* y, double rr, double dr, double stp, double dtd) {
        const int l = lane_id();
        if (iupdat <= QB_DS_M) {
            col = iupdat;
            tail = (head + iupdat - 1) % QB_DS_M;
        } else {
            tail = (tail + 1) % QB_DS_M;
            head = (head + 1) % QB_DS_M;
        }
        if (l < n) {
            w.ws[l + QB_DS_N * tail] = s[l];
            w.wy[l + QB_DS_N * tail] = y[l];
        }
        theta = rr / dr;
        if (iupdat > QB_DS_M) {   // drop the oldest pair: shift SS (upper) and SY (lower) up-left
            const int c1 = col - 1;
            double* tmp = w.wn;   // free until the next form_k
            for (int e = l; e < c1 * c1; e += 32) {
                const int i = e % c1, j = e / c1;
                tmp[e] = (i <= j) ? SS(i + 1, j + 1) : 0.0;
                tmp[c1 * c1 + e] = (i >= j) ? SY(i + 1, j + 1) : 0.0;
            }
            __syncwarp();
            for (int e = l; e < c1 * c1; e += 32) {
                const int i = e % c1, j = e / c1;
                if (i <= j) SS(i, j) = tmp[e];
                if (i >= j) SY(i, j) = tmp[c1 * c1 + e];
            }
        }
        __syncwarp();
        if (l < col - 1) {
            const double *yj = ycol(l), *sj = scol(l);
            double a = 0, b = 0;
            for (int i = 0; i < n; ++i) {
                a = fma(s[i], yj[i], a);
                b = fma(sj[i], s[i], b);
            }
            SY(col - 1, l) = a;
            SS(l, col - 1) = b;
        }
        if (l == 0) {
            SS(col - 1, col - 1) = (stp == 1.0) ? dtd : stp * stp * dtd;
            SY(col - 1, col - 1) = dr;
        }
        __syncwarp();
    }

    // Minimise from w.x (in place); factr 1e5, pgtol 1e-15, 10000 iterations / evaluations.
    __device__ int run() {
        const double tol = 1e5 * kEps, pgtol = 1e-15;
        const int maxiter = 10000, maxfun = 10000;
        const int l = lane_id();
        const bool own = l < n;
        double *x = w.x, *g = w.g, *z = w.z, *d = w.d, *r = w.r, *xs = w.xs, *gs = w.gs;
        if (own) {
            if (bounded && x[l] < 0.0) x[l] = 0.0;
            w.where[l] = bounded ? 0 : -1;
        }
        nfree = 0;
        __syncwarp();
        double f = fg(w, n, x, g);
        int nfgv = 1, iter = 0;
        if (pg_norm(x, g) <= pgtol) return iter;
        for (int outer = 0; outer < 4 * maxiter; ++outer) {
            if (!bounded && col > 0) {
                if (own) z[l] = x[l];
                __syncwarp();
            } else {
                if (cauchy(x, g, z, w.cw) != 0) { refresh(); continue; }
                collect_free();
            }
            if (nfree > 0 && col > 0) {
                if (form_k() != 0) { refresh(); continue; }
                if (reduced_gradient(x, g, z, w.cw, r) != 0) { refresh(); continue; }
                if (subspace_min(x, g, z, r) != 0) { refresh(); continue; }
            }
            double dl = own ? z[l] - x[l] : 0.0;
            if (own) d[l] = dl;
            const double dtd = wsum(dl * dl);
            const double dnorm = sqrt(dtd);
            __syncwarp();
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
            const double xl0 = own ? x[l] : 0.0, gl0 = own ? g[l] : 0.0;
            if (own) {
                xs[l] = xl0;
                gs[l] = gl0;
            }
            const double fold = f;
            int ifun = 0, iback = 0;
            double gd = 0, gdold = 0;
            Search S;
            bool newx = false, start = true;
            for (int ls = 0; ls < 64; ++ls) {
                gd = wsum(own ? g[l] * dl : 0.0);
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
                    __syncwarp();
                    if (own) x[l] = (stp == 1.0) ? z[l] : fma(stp, dl, xl0);
                    __syncwarp();
                    if (iback >= 20) break;
                    f = fg(w, n, x, g);
                    continue;
                }
                newx = true;
                break;
            }
            if (!newx) {
                __syncwarp();
                if (own) {
                    x[l] = xl0;
                    g[l] = gl0;
                }
                __syncwarp();
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
            const double rl = own ? g[l] - gl0 : 0.0;
            if (own) r[l] = rl;
            const double rr = wsum(rl * rl);
            double dr, ddum;
            if (stp == 1.0) {
                dr = gd - gdold;
                ddum = -gdold;
            } else {
                dr = (gd - gdold) * stp;
                if (own) d[l] = dl * stp;
                ddum = -gdold * stp;
            }
            __syncwarp();
            if (dr <= kEps * ddum) continue;
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
    const int l = lane_id();
    const bool own = l < n;
    double *x = w.x, *g = w.g, *xn = w.z, *gn = w.r;
    auto pg_norm = [&]() {
        double t = 0.0;
        if (own) {
            t = x[l] - g[l];
            if (bounded) t = fmax(t, 0.0);
            t = fabs(t - x[l]);
        }
        return wmax(t);
    };
    if (bounded && own) x[l] = fmax(x[l], 0.0);
    __syncwarp();
    double fc = obj_f(w, n, x);
    obj_g(w, n, x, g);
    int nfeval = 1, nit = 0;
    double gnorm = pg_norm();
    if (gnorm <= eps) return 0;
    if (l < mem) w.fprev[l] = fc;
    double lam = fmin(lmax, fmax(lmin, 1.0 / gnorm));
    while (nit < nitmax) {
        double dl = 0.0, xl = 0.0, gl = 0.0;
        if (own) {
            xl = x[l];
            gl = g[l];
            double t = xl - lam * gl;
            if (bounded) t = fmax(t, 0.0);
            dl = t - xl;
        }
        const double gtd = wsum(gl * dl);
        __syncwarp();
        const double fref = wmax(l < mem ? w.fprev[l] : -INFINITY);
        double alpha = 1.0;
        if (own) xn[l] = fma(alpha, dl, xl);
        __syncwarp();
        double fn = obj_f(w, n, xn);
        ++nfeval;
        while (fn > fref + gamma * alpha * gtd) {
            const double atemp = -0.5 * gtd * alpha * alpha / (fn - fc - alpha * gtd);
            if (atemp >= sigma1 && atemp <= sigma2 * alpha) alpha = atemp;
            else alpha /= 2;
            __syncwarp();
            if (own) xn[l] = fma(alpha, dl, xl);
            __syncwarp();
            fn = obj_f(w, n, xn);
            if (++nfeval > nfevalmax) {
                if (own) x[l] = xn[l];
                __syncwarp();
                return 2;
            }
        }
        ++nit;
        __syncwarp();
        if (l == 0) w.fprev[nit % mem] = fn;
        obj_g(w, n, xn, gn);
        double s = 0.0, y = 0.0;
        if (own) {
            s = xn[l] - xl;
            y = gn[l] - gl;
        }
        const double sts = wsum(s * s), sty = wsum(s * y);
        lam = sty <= 0 ? lmax : fmin(lmax, fmax(lmin, sts / sty));
        if (own) {
            x[l] = xn[l];
            g[l] = gn[l];
        }
        __syncwarp();
        fc = fn;
        gnorm = pg_norm();
        if (gnorm <= eps) return 0;
    }
    return 1;
}

// LU with partial pivoting of the leading n x n block of A (column-major, leading dimension
// n, n <= 32), solving A x = b in place of b; returns the determinant (0 when a pivot
// vanishes).  Lane i owns row i in the elimination.
__device__ inline double lu_solve(int n, double* A, double* b) {
    const int l = lane_id();
    double det = 1.0;
    __syncwarp();
    for (int k = 0; k < n; ++k) {
        const bool cand = l >= k && l < n;
        const double a = cand ? fabs(A[l + n * k]) : -1.0;
        const double mx = wmax(a);
        const int p = __ffs(__ballot_sync(kFull, cand && a == mx)) - 1;   // first largest
        if (A[p + n * k] == 0.0) return 0.0;
        __syncwarp();
        if (p != k) {
            if (l < n) {
                const double t = A[k + n * l];
                A[k + n * l] = A[p + n * l];
                A[p + n * l] = t;
            }
            if (l == 0) {
                const double t = b[k];
                b[k] = b[p];
                b[p] = t;
            }
            det = -det;
            __syncwarp();
        }
        const double pv = A[k + n * k];
        det *= pv;
        if (l > k && l < n) {
            const double f = A[l + n * k] / pv;
            A[l + n * k] = f;
            for (int j = k + 1; j < n; ++j) A[l + n * j] = fma(-f, A[k + n * j], A[l + n * j]);
            b[l] = fma(-f, b[k], b[l]);
        }
        __syncwarp();
    }
    const double rl = l < n ? 1.0 / A[l + n * l] : 0.0;
    double bl = l < n ? b[l] : 0.0;
    for (int i = n - 1; i >= 0; --i) {
        if (l == i) bl *= rl;
        const double bi = __shfl_sync(kFull, bl, i);
        if (l < i) bl = fma(-A[l + n * i], bi, bl);
    }
    __syncwarp();
    if (l < n) b[l] = bl;
    __syncwarp();
    return det;
}

}  // namespace qbds

// CMsolver! (HartreeFock.jl:1445-1477) by one warp: solve [B 1; 1 0][c; l] = [-v; 1]; if
// `convex` and some c < 0, try the subsystems with index subsets removed (by increasing
// size, smallest |c| first) until a non-negative solution appears; a singular bordered
// matrix gets B += 4e-13 I (1000 getAtolVal).  B is m x m with leading dimension ldb, m <= 16.
// Bounded: at most 64 perturbation rounds; returns false if they run out (c then holds the
// last candidate).  Every lane walks the subsets alike; the LU solves are spread over lanes.
static __device__ __noinline__ bool qb_cm_solve(QbDiisWork& w, int m, int convex, const double* Bin, int ldb,
                                                const double* v, double* c) {
    const int M = m + 1, l = qbds::lane_id();
    double *B = w.cmB, *A = w.cmA, *W = w.cmW, *b = w.cmb, *x = w.cmx;
    for (int e = l; e < m * m; e += 32) B[e] = Bin[(e % m) + ldb * (e / m)];
    __syncwarp();
    for (int round = 0; round < 64; ++round) {
        for (int guard = 0; guard < 64; ++guard) {
            for (int e = l; e < M * M; e += 32) {
                const int i = e % M, j = e / M;
                const double a = (i < m && j < m) ? B[i + m * j] : ((i == m && j == m) ? 0.0 : 1.0);
                A[e] = a;
                W[e] = a;
            }
            if (l < M) x[l] = 0.0;
            if (qbds::lu_solve(M, W, x) != 0.0) break;
            if (l < m) B[l + m * l] += 4e-13;
            __syncwarp();
        }
        if (l < m) b[l] = v ? -v[l] : 0.0;
        if (l == m) b[l] = 1.0;
        for (int e = l; e < M * M; e += 32) W[e] = A[e];
        __syncwarp();
        if (l < M) x[l] = b[l];
        qbds::lu_solve(M, W, x);
        const double xl = l < m ? x[l] : 0.0;
        if (l < m) c[l] = xl;
        const bool neg = qbds::wany(l < m && xl < 0.0);
        if (!convex || !neg) {
            __syncwarp();
            return true;
        }
        int perm[QB_DS_N];
        for (int i = 0; i < m; ++i) perm[i] = i;
        for (int i = 1; i < m; ++i) {   // stable insertion sort by |c|
            const int t = perm[i];
            int j = i - 1;
            while (j >= 0 && fabs(x[perm[j]]) > fabs(x[t])) {
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
                __syncwarp();
                if (l < k) {
                    const int kl = keep[l];
                    x[l] = b[kl];
                    for (int jj = 0; jj < k; ++jj) W[l + k * jj] = A[kl + M * keep[jj]];
                }
                if (qbds::lu_solve(k, W, x) != 0.0) {
                    const double xk = l < k - 1 ? x[l] : 0.0;
                    if (l < m) c[l] = 0.0;
                    __syncwarp();
                    if (l < k - 1) c[keep[l]] = xk;
                    __syncwarp();
                    if (!qbds::wany(l < k - 1 && xk < 0.0)) return true;
                }
                int pos = sz - 1;
                while (pos >= 0 && comb[pos] == m - sz + pos) --pos;
                if (pos < 0) break;
                ++comb[pos];
                for (int t = pos + 1; t < sz; ++t) comb[t] = comb[t - 1] + 1;
            }
        }
        if (l < m) B[l + m * l] += 4e-13;
        __syncwarp();
    }
    return false;
}

// One warp: solve the DIIS coefficient problem of m entries.  B (m x m, leading dimension
// ldb) and v (m) describe it; c (m) is the starting point on entry and the normalised
// coefficients on return.  solver: QB_DIIS_LBFGS or QB_DIIS_SPGB; convex adds c >= 0.
// Returns the solver's iteration count (L-BFGS-B) or status (SPG).
static __device__ __noinline__ int qb_diis_iterative_solve(QbDiisWork& w, int solver, int convex, int m, const double* B,
                                                           int ldb, const double* v, double* c) {
    const int l = qbds::lane_id();
    for (int e = l; e < m * m; e += 32) w.B[(e % m) + QB_DS_N * (e / m)] = B[(e % m) + ldb * (e / m)];
    if (l < m) {
        w.v[l] = v ? v[l] : 0.0;
        w.x[l] = c[l];
    }
    __syncwarp();
    int out;
    if (solver == QB_DIIS_SPGB) {
        out = qbds::spg(w, m, convex != 0);
    } else {
        qbds::Lbfgsb opt(w, m, convex != 0);
        out = opt.run();
    }
    if (l == 0) w.iters = out;
    const double s = qbds::shifted_sum(m, w.x);
    if (l < m) c[l] = w.x[l] / s;
    __syncwarp();
    return out;
}
