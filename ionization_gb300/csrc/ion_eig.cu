// Eigenpairs of batched real symmetric tridiagonal matrices: the numeric
// eigenstate basis of the spherical-harmonic and line meshes
// (SphericalHarmonicMesh.get_numeric_eigenstate_basis, ionization/mesh/
// meshes.py:1281-1356, and LineMesh._get_numeric_eigenstate_basis,
// meshes.py:343-387), which the reference finds with scipy's Lanczos eigsh on
// each single-l (or the line's) field-free Hamiltonian.
//
// Here every eigenpair is independent work:
//   ion_tridiag_count_below  Sturm count of the eigenvalues below x, one
//                            thread per matrix;
//   ion_tridiag_eigvals      the k-th smallest eigenvalue by bisection on the
//                            Sturm count (Gershgorin bracket, to the last
//                            bits of FP64), one thread per requested pair;
//   ion_tridiag_eigvecs      inverse iteration, one thread per requested
//                            pair: Gaussian elimination with partial pivoting
//                            of T - lambda I (two solves from a fixed
//                            pseudo-random start), unit 2-norm, sign fixed
//                            so that the first component above 1e-3 of the
//                            largest is positive.
// The factors live in device scratch interleaved by request, so the threads
// of a warp touch consecutive addresses.
#include "ion_common.cuh"

namespace ion {

__device__ __forceinline__ double sq(double v) { return v * v; }

// number of eigenvalues of T (diag d, off e) below x (LDL^T inertia)
__device__ int sturm_count(const double* d, const double* e, int n, double x, double pivmin) {
    int count = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) ++count;
    for (int k = 1; k < n; ++k) {
        q = (d[k] - x) - sq(e[k - 1]) / q;
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0.0) ++count;
    }
    return count;
}

__device__ double tridiag_pivmin(const double* e, int n) {
    double m = 1.0;
    for (int k = 0; k + 1 < n; ++k) m = fmax(m, sq(e[k]));
    return 1e-290 * m;  // a safe minimum pivot, scaled as LAPACK's dstebz scales it
}

__global__ void tridiag_count_kernel(int n_mat, int n, const double* diag, const double* off, const double* x,
                                     int32_t* counts) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n_mat) return;
    const double* d = diag + int64_t(m) * n;
    const double* e = off + int64_t(m) * (n - 1);
    counts[m] = sturm_count(d, e, n, x[m], tridiag_pivmin(e, n));
}

__global__ void tridiag_eigvals_kernel(int n_mat, int n, const double* diag, const double* off, int n_req,
                                       const int32_t* req_mat, const int32_t* req_idx, double* vals) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_req) return;
    const int m = req_mat[r], idx = req_idx[r];
    if (m < 0 || m >= n_mat || idx < 0 || idx >= n) {
        vals[r] = nan("");
        return;
    }
    const double* d = diag + int64_t(m) * n;
    const double* e = off + int64_t(m) * (n - 1);
    double lo = d[0], hi = d[0];
    for (int k = 0; k < n; ++k) {
        const double rad = (k > 0 ? fabs(e[k - 1]) : 0.0) + (k + 1 < n ? fabs(e[k]) : 0.0);
        lo = fmin(lo, d[k] - rad);
        hi = fmax(hi, d[k] + rad);
    }
    const double widen = 4.0 * n * 2.220446049250313e-16 * fmax(fabs(lo), fabs(hi)) + 1e-300;
    lo -= widen;
    hi += widen;
    const double pivmin = tridiag_pivmin(e, n);
    // invariant: count(lo) <= idx < count(hi)
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;  // the bracket is two adjacent doubles
        if (sturm_count(d, e, n, mid, pivmin) > idx)
            hi = mid;
        else
            lo = mid;
    }
    vals[r] = 0.5 * (lo + hi);
}

// scratch field f of row k of request r
__device__ __forceinline__ double& scr(double* s, int f, int k, int n, int n_req, int r) {
    return s[(int64_t(f) * n + k) * n_req + r];
}

__global__ void tridiag_eigvecs_kernel(int n_mat, int n, const double* diag, const double* off, int n_req,
                                       const int32_t* req_mat, const double* vals, double* vecs, double* s) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n_req) return;
    const int m = req_mat[r];
    double* out = vecs + int64_t(r) * n;
    if (m < 0 || m >= n_mat || !(vals[r] == vals[r])) {
        for (int k = 0; k < n; ++k) out[k] = nan("");
        return;
    }
    const double* d = diag + int64_t(m) * n;
    const double* e = off + int64_t(m) * (n - 1);
    const double lam = vals[r];
    // factor T - lam I = P L U; U has diagonal D, super S, second super S2
    enum { FD = 0, FS = 1, FS2 = 2, FL = 3, FP = 4, FX = 5 };
    double scale = 0.0;
    for (int k = 0; k < n; ++k) scale = fmax(scale, fabs(d[k] - lam) + (k + 1 < n ? fabs(e[k]) : 0.0));
    const double tiny = fmax(scale, 1e-300) * 2.220446049250313e-16;
    for (int k = 0; k < n; ++k) {
        scr(s, FD, k, n, n_req, r) = d[k] - lam;
        scr(s, FS, k, n, n_req, r) = k + 1 < n ? e[k] : 0.0;
        scr(s, FS2, k, n, n_req, r) = 0.0;
    }
    for (int k = 0; k + 1 < n; ++k) {
        double dk = scr(s, FD, k, n, n_req, r);
        const double sub = e[k];  // entry (k+1, k), untouched by earlier steps
        if (fabs(dk) >= fabs(sub)) {
            if (dk == 0.0) dk = tiny;
            const double mlt = sub / dk;
            scr(s, FD, k, n, n_req, r) = dk;
            scr(s, FL, k, n, n_req, r) = mlt;
            scr(s, FP, k, n, n_req, r) = 0.0;
            scr(s, FD, k + 1, n, n_req, r) -= mlt * scr(s, FS, k, n, n_req, r);
        } else {  // swap rows k and k+1
            const double mlt = dk / sub;
            const double sk = scr(s, FS, k, n, n_req, r);
            const double d1 = scr(s, FD, k + 1, n, n_req, r);
            const double s1 = scr(s, FS, k + 1, n, n_req, r);
            scr(s, FD, k, n, n_req, r) = sub;
            scr(s, FS, k, n, n_req, r) = d1;
            scr(s, FS2, k, n, n_req, r) = s1;
            scr(s, FD, k + 1, n, n_req, r) = sk - mlt * d1;
            scr(s, FS, k + 1, n, n_req, r) = -mlt * s1;
            scr(s, FL, k, n, n_req, r) = mlt;
            scr(s, FP, k, n, n_req, r) = 1.0;
        }
    }
    if (scr(s, FD, n - 1, n, n_req, r) == 0.0) scr(s, FD, n - 1, n, n_req, r) = tiny;
    // start: a fixed pseudo-random vector in [0.5, 1.5)
    uint32_t h = 0x9e3779b9u ^ uint32_t(r * 2654435761u);
    for (int k = 0; k < n; ++k) {
        h ^= h << 13;
        h ^= h >> 17;
        h ^= h << 5;
        scr(s, FX, k, n, n_req, r) = 0.5 + double(h) * (1.0 / 4294967296.0);
    }
    for (int pass = 0; pass < 2; ++pass) {
        for (int k = 0; k + 1 < n; ++k) {  // forward: P and L
            const double mlt = scr(s, FL, k, n, n_req, r);
            double& b0 = scr(s, FX, k, n, n_req, r);
            double& b1 = scr(s, FX, k + 1, n, n_req, r);
            if (scr(s, FP, k, n, n_req, r) == 0.0) {
                b1 -= mlt * b0;
            } else {
                const double t = b0;
                b0 = b1;
                b1 = t - mlt * b0;
            }
        }
        for (int k = n - 1; k >= 0; --k) {  // back substitution with U
            double v = scr(s, FX, k, n, n_req, r);
            if (k + 1 < n) v -= scr(s, FS, k, n, n_req, r) * scr(s, FX, k + 1, n, n_req, r);
            if (k + 2 < n) v -= scr(s, FS2, k, n, n_req, r) * scr(s, FX, k + 2, n, n_req, r);
            scr(s, FX, k, n, n_req, r) = v / scr(s, FD, k, n, n_req, r);
        }
        double big = 0.0;
        for (int k = 0; k < n; ++k) big = fmax(big, fabs(scr(s, FX, k, n, n_req, r)));
        double nrm = 0.0;
        for (int k = 0; k < n; ++k) nrm += sq(scr(s, FX, k, n, n_req, r) / big);
        const double inv = 1.0 / (big * sqrt(nrm));
        for (int k = 0; k < n; ++k) scr(s, FX, k, n, n_req, r) *= inv;
    }
    double big = 0.0;
    for (int k = 0; k < n; ++k) big = fmax(big, fabs(scr(s, FX, k, n, n_req, r)));
    double sign = 1.0;
    for (int k = 0; k < n; ++k) {
        const double v = scr(s, FX, k, n, n_req, r);
        if (fabs(v) > 1e-3 * big) {
            sign = v < 0.0 ? -1.0 : 1.0;
            break;
        }
    }
    for (int k = 0; k < n; ++k) out[k] = sign * scr(s, FX, k, n, n_req, r);
}

static int eig_args_ok(int n_mat, int n, const void* diag, const void* off) {
    if (n_mat < 0 || n < 2 || (n_mat > 0 && (!diag || !off))) {
        set_error("ion_tridiag: invalid argument");
        return 0;
    }
    return 1;
}

}  // namespace ion

using namespace ion;

extern "C" {
int64_t ion_tridiag_eig_scratch_doubles(int32_t n, int32_t n_req) { return int64_t(6) * n * n_req; }

int ion_tridiag_count_below(int32_t n_mat, int32_t n, const double* diag, const double* off, const double* x,
                            int32_t* counts, void* stream) {
    if (!eig_args_ok(n_mat, n, diag, off) || (n_mat > 0 && (!x || !counts))) return ION_ERR_INVALID_ARGUMENT;
    if (n_mat == 0) return ION_OK;
    tridiag_count_kernel<<<(n_mat + 127) / 128, 128, 0, as_stream(stream)>>>(n_mat, n, diag, off, x, counts);
    return check_launch("tridiag_count_kernel");
}

int ion_tridiag_eigvals(int32_t n_mat, int32_t n, const double* diag, const double* off, int32_t n_req,
                        const int32_t* req_mat, const int32_t* req_idx, double* vals, void* stream) {
    if (!eig_args_ok(n_mat, n, diag, off) || n_req < 0 || (n_req > 0 && (!req_mat || !req_idx || !vals)))
        return ION_ERR_INVALID_ARGUMENT;
    if (n_req == 0) return ION_OK;
    tridiag_eigvals_kernel<<<(n_req + 63) / 64, 64, 0, as_stream(stream)>>>(n_mat, n, diag, off, n_req, req_mat,
                                                                            req_idx, vals);
    return check_launch("tridiag_eigvals_kernel");
}

int ion_tridiag_eigvecs(int32_t n_mat, int32_t n, const double* diag, const double* off, int32_t n_req,
                        const int32_t* req_mat, const double* vals, double* vecs, double* scratch, void* stream) {
    if (!eig_args_ok(n_mat, n, diag, off) || n_req < 0 ||
        (n_req > 0 && (!req_mat || !vals || !vecs || !scratch)))
        return ION_ERR_INVALID_ARGUMENT;
    if (n_req == 0) return ION_OK;
    tridiag_eigvecs_kernel<<<(n_req + 63) / 64, 64, 0, as_stream(stream)>>>(n_mat, n, diag, off, n_req, req_mat,
                                                                            vals, vecs, scratch);
    return check_launch("tridiag_eigvecs_kernel");
}
}
