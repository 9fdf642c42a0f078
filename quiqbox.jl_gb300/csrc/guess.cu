// Learned initial guess: atom-pair features and density assembly on the device.
//
// The network (csrc/mlp.cu) maps one atom pair (A, B), A <= B, of a minimal-basis
// (STO-3G, H/C/N/O) molecule to the 5 x 5 block of the converged per-spin density between
// A's and B's functions, written in a local frame of the pair; these two kernels produce
// its input rows and turn its output rows back into per-molecule densities, the
// initial-density input of the batched SCF.  One thread per pair, every atom of the
// pair's molecule visited in a loop (molecules are small).  Geometry runs in FP64; the
// features are rounded to FP32 once, at the end.
//
// Local frame: for A != B, z along A -> B and x towards the atom nearest the bond midpoint
// (its component perpendicular to z, at least 0.3 bohr); for A == B, z towards A's
// nearest neighbour and x towards the nearest other atom with a perpendicular component of
// at least 0.3 bohr.  Without such an atom x is a fixed unit vector perpendicular to z;
// y = z x x.  Features (row of 128 floats, 74 used): 32 Gaussians exp(-((r - mu_k) / 0.25)^2)
// of r = |AB|, mu_k = 0.25 (k + 1); the same-atom flag; element one-hots of A and B; per
// endpoint P in (A, B) and per element e of the other atoms i != P, the sums of
// w (1, cos_z, cos_x, (3 cos_z^2 - 1) / 2), w = exp(-(|r_iP| / 2.5)^2), in the local frame;
// the molecular charge.
#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>
#include "qb_internal.h"

namespace {

constexpr int kFeatStride = 128;
constexpr int kEnv = 41;

__device__ __forceinline__ double3 sub3(double3 a, double3 b) { return make_double3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ double dot3(double3 a, double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ double3 scale3(double3 a, double s) { return make_double3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ double3 cross3(double3 a, double3 b) {
    return make_double3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ double3 unit3(double3 a) { return scale3(a, 1.0 / fmax(sqrt(dot3(a, a)), 1e-300)); }
__device__ __forceinline__ double3 load3(const double* p, int i) {
    return make_double3(p[3 * i], p[3 * i + 1], p[3 * i + 2]);
}

// Local frame (x, y, z) of pair (a, b), atoms [a0, a0 + na) of its molecule.
__device__ void pair_frame(int a, int b, int a0, int na, const double* __restrict__ pos, double3& x, double3& y,
                           double3& z) {
    const double3 PA = load3(pos, a), PB = load3(pos, b);
    const bool same = a == b;
    int n1 = -1;
    double best = INFINITY;
    for (int i = a0; i < a0 + na; ++i) {
        if (i == a) continue;
        const double3 u = sub3(load3(pos, i), PA);
        const double d = sqrt(dot3(u, u));
        if (d < best) {
            best = d;
            n1 = i;
        }
    }
    if (!same) z = unit3(sub3(PB, PA));
    else if (n1 >= 0) z = unit3(sub3(load3(pos, n1), PA));
    else z = make_double3(0.0, 0.0, 1.0);
    const double3 mid = scale3(make_double3(PA.x + PB.x, PA.y + PB.y, PA.z + PB.z), 0.5);
    double bestc = INFINITY;
    double3 xr = make_double3(0.0, 0.0, 0.0);
    bool has_ref = false;
    for (int i = a0; i < a0 + na; ++i) {
        if (i == a || (!same && i == b) || (same && i == n1)) continue;
        const double3 Pi = load3(pos, i);
        const double3 rel = sub3(Pi, PA);
        const double3 perp = sub3(rel, scale3(z, dot3(rel, z)));
        if (!(sqrt(dot3(perp, perp)) > 0.3)) continue;
        const double3 v = same ? rel : sub3(Pi, mid);
        const double key = sqrt(dot3(v, v));
        if (key < bestc) {
            bestc = key;
            xr = perp;
            has_ref = true;
        }
    }
    if (has_ref) {
        x = unit3(xr);
    } else {
        const double3 helper = fabs(z.z) < 0.9 ? make_double3(0.0, 0.0, 1.0) : make_double3(1.0, 0.0, 0.0);
        x = unit3(cross3(helper, z));
    }
    y = cross3(z, x);
}

__global__ void qb_guess_features_kernel(int npair, const int* __restrict__ pair_mol, const int* __restrict__ pair_a,
                                         const int* __restrict__ pair_b, const int* __restrict__ mol_atom0,
                                         const int* __restrict__ mol_natom, const double* __restrict__ pos,
                                         const int* __restrict__ el, const float* __restrict__ charge,
                                         float* __restrict__ X, double* __restrict__ R) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npair) return;
    const int m = pair_mol[p], a = pair_a[p], b = pair_b[p];
    const int a0 = mol_atom0[m], na = mol_natom[m];
    double3 x, y, z;
    pair_frame(a, b, a0, na, pos, x, y, z);
    double* Rp = R + 9 * (size_t)p;   // R[i][j] (row-major) = component i of local axis j
    Rp[0] = x.x; Rp[1] = y.x; Rp[2] = z.x;
    Rp[3] = x.y; Rp[4] = y.y; Rp[5] = z.y;
    Rp[6] = x.z; Rp[7] = y.z; Rp[8] = z.z;
    float* row = X + (size_t)p * kFeatStride;
    const double3 PA = load3(pos, a), PB = load3(pos, b);
    const double3 ab = sub3(PB, PA);
    const double r = sqrt(dot3(ab, ab));
    for (int k = 0; k < 32; ++k) {
        const double t = (r - (0.25 + 0.25 * k)) / 0.25;
        row[k] = (float)exp(-t * t);
    }
    row[32] = a == b ? 1.0f : 0.0f;
    for (int k = 33; k < kEnv; ++k) row[k] = 0.0f;
    row[33 + el[a]] = 1.0f;
    row[37 + el[b]] = 1.0f;
    for (int e_off = 0; e_off < 2; ++e_off) {
        const int me = e_off ? b : a;
        const double3 P = e_off ? PB : PA;
        double acc[16];
        for (int k = 0; k < 16; ++k) acc[k] = 0.0;
        for (int i = a0; i < a0 + na; ++i) {
            if (i == me) continue;
            const double3 u = sub3(load3(pos, i), P);
            const double d = sqrt(dot3(u, u));
            const double w = exp(-(d / 2.5) * (d / 2.5));
            const double dn = fmax(d, 1e-12);
            const double cz = dot3(u, z) / dn, cx = dot3(u, x) / dn;
            double* t = acc + 4 * el[i];
            t[0] += w;
            t[1] += w * cz;
            t[2] += w * cx;
            t[3] += w * 0.5 * (3.0 * cz * cz - 1.0);
        }
        for (int k = 0; k < 16; ++k) row[kEnv + 16 * e_off + k] = (float)acc[k];
    }
    row[73] = charge[m];
    for (int k = 74; k < kFeatStride; ++k) row[k] = 0.0f;
}

// Density of the pair's block in the lab frame, blk = T loc T^T with T = diag(1, 1, R)
// (functions 1s, 2s, 2px, 2py, 2pz; H uses the first only), symmetrised for A == B, and
// written to both (A, B) and (B, A) of the molecule's column-major density.
__global__ void qb_guess_assemble_kernel(int npair, const int* __restrict__ pair_mol, const int* __restrict__ pair_a,
                                         const int* __restrict__ pair_b, const int* __restrict__ el,
                                         const int* __restrict__ atom_f0, const long long* __restrict__ mol_off,
                                         const int* __restrict__ mol_n, const float* __restrict__ Y, int ldy,
                                         const double* __restrict__ R, double* __restrict__ D) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npair) return;
    const int m = pair_mol[p], a = pair_a[p], b = pair_b[p];
    const int n = mol_n[m];
    double* Dm = D + mol_off[m];
    double T[5][5];
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 5; ++j) T[i][j] = (i == j && i < 2) ? 1.0 : 0.0;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[2 + i][2 + j] = R[9 * (size_t)p + 3 * i + j];
    const float* loc = Y + (size_t)p * ldy;
    double tl[5][5], blk[5][5];
    for (int i = 0; i < 5; ++i)
        for (int k = 0; k < 5; ++k) {
            double s = 0.0;
            for (int j = 0; j < 5; ++j) s += T[i][j] * (double)loc[5 * j + k];
            tl[i][k] = s;
        }
    for (int i = 0; i < 5; ++i)
        for (int l = 0; l < 5; ++l) {
            double s = 0.0;
            for (int k = 0; k < 5; ++k) s += tl[i][k] * T[l][k];
            blk[i][l] = s;
        }
    if (a == b)
        for (int i = 0; i < 5; ++i)
            for (int l = i + 1; l < 5; ++l) {
                const double v = 0.5 * (blk[i][l] + blk[l][i]);
                blk[i][l] = v;
                blk[l][i] = v;
            }
    const int na = el[a] == 0 ? 1 : 5, nb = el[b] == 0 ? 1 : 5;
    const int fa = atom_f0[a], fb = atom_f0[b];
    for (int i = 0; i < na; ++i)
        for (int j = 0; j < nb; ++j) {
            Dm[(fa + i) + (size_t)n * (fb + j)] = blk[i][j];
            Dm[(fb + j) + (size_t)n * (fa + i)] = blk[i][j];
        }
}

}  // namespace

extern "C" {

int qb_guess_features(int npair, const int* pair_mol, const int* pair_a, const int* pair_b, const int* mol_atom0,
                      const int* mol_natom, const double* atom_pos, const int* atom_el, const float* mol_charge,
                      float* X, double* R, void* stream) {
    if (npair < 0) return QB_ERR_DIM;
    if (npair == 0) return QB_OK;
    if (!pair_mol || !pair_a || !pair_b || !mol_atom0 || !mol_natom || !atom_pos || !atom_el || !mol_charge || !X ||
        !R)
        return QB_ERR_ARG;
    qb_guess_features_kernel<<<(npair + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        npair, pair_mol, pair_a, pair_b, mol_atom0, mol_natom, atom_pos, atom_el, mol_charge, X, R);
    return cudaGetLastError() == cudaSuccess ? QB_OK : QB_ERR_CUDA;
}

int qb_guess_assemble(int npair, const int* pair_mol, const int* pair_a, const int* pair_b, const int* atom_el,
                      const int* atom_f0, const long long* mol_off, const int* mol_n, const float* Y, int ldy,
                      const double* R, double* D, void* stream) {
    if (npair < 0 || ldy < 25) return QB_ERR_DIM;
    if (npair == 0) return QB_OK;
    if (!pair_mol || !pair_a || !pair_b || !atom_el || !atom_f0 || !mol_off || !mol_n || !Y || !R || !D)
        return QB_ERR_ARG;
    qb_guess_assemble_kernel<<<(npair + 127) / 128, 128, 0, static_cast<cudaStream_t>(stream)>>>(
        npair, pair_mol, pair_a, pair_b, atom_el, atom_f0, mol_off, mol_n, Y, ldy, R, D);
    return cudaGetLastError() == cudaSuccess ? QB_OK : QB_ERR_CUDA;
}

}  // extern "C"
