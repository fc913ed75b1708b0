// Block-cooperative tridiagonal line solver.
//
// One line (a tridiagonal system of n rows) is solved by T threads of a CTA.
// Thread t owns a contiguous chunk of m >= 2 rows [s, s+m).  The method is the
// partition method (H. H. Wang, "A parallel method for tridiagonal
// equations", ACM TOMS 7(2), 1981) followed by parallel cyclic reduction
// (R. W. Hockney, 1965; Hockney & Jesshope) on the reduced system:
//
//  1. chunk elimination (registers): the interior rows s+1..e-1 are solved
//     with x_s and x_e as parameters,  x_i = alpha_i + beta_i x_s + gamma_i x_e,
//     by one forward and one backward Thomas pass over the chunk;
//  2. substituting x_{s+1} and x_{e-1} into the chunk's first and last rows
//     gives two equations per chunk coupling only chunk end points: a
//     tridiagonal system of 2T unknowns ordered (s_0, e_0, s_1, e_1, ...);
//  3. that system is solved by PCR in shared memory, each row normalised so
//     its diagonal is 1 (one complex reciprocal per row per level);
//  4. each thread expands its interior rows from alpha, beta, gamma.
//
// Coefficients come from a functor ``coef(i, a, b, c)`` returning A[i,i-1],
// A[i,i], A[i,i+1]; it must return a = 0 on row 0 and c = 0 on row n-1.  The
// right-hand side comes from ``rhs(i)`` and the solution leaves through
// ``out(i, x_i)``.  Every thread of the CTA must call block_line_solve
// (``active`` = false for idle threads) because it uses __syncthreads().
#pragma once

#include "ion_common.cuh"

namespace ion {

__host__ __device__ __forceinline__ void chunk_bounds(int64_t n, int64_t T, int64_t t, int64_t& s,
                                                      int& m) {
    int64_t base = n / T;
    int64_t rem = n - base * T;
    s = t * base + (t < rem ? t : rem);
    m = int(base + (t < rem ? 1 : 0));
}

// shared memory (bytes) used by one line's PCR: A, C, D double-buffered
template <typename R>
__host__ __device__ constexpr size_t pcr_smem_bytes(int T) {
    return 6 * 2 * size_t(T) * sizeof(Cx<R>);
}

__host__ __device__ __forceinline__ int pcr_levels(int N) {
    int L = 0;
    while ((1 << L) < N) ++L;
    return L;
}

// Normalised reduced row:  a x_{k-1} + x_k + c x_{k+1} = d
template <typename R>
struct RedRow {
    Cx<R> a, c, d;
};

// Phase 1+2 for the chunk [s, s+m): fills alpha/beta/gamma for interior rows
// k = 1..m-2 (indices relative to s) and returns the chunk's two normalised
// reduced rows.
template <typename R, int MAXM, class Coef, class Rhs>
__device__ __forceinline__ void chunk_eliminate(int64_t s, int m, const Coef& coef, const Rhs& rhs,
                                                Cx<R> (&al)[MAXM], Cx<R> (&be)[MAXM],
                                                Cx<R> (&ga)[MAXM], RedRow<R>& rowS,
                                                RedRow<R>& rowE) {
    const Cx<R> zero = {R(0), R(0)};
#pragma unroll
    for (int k = 0; k < MAXM; ++k) {
        al[k] = zero;
        be[k] = zero;
        ga[k] = zero;
    }
    const Cx<R> y0 = rhs(s);
    const Cx<R> yl = rhs(s + m - 1);

    // forward pass over interior rows k = 1..m-2
    Cx<R> cprev = zero, daprev = zero, dbprev = zero, glast = zero;
#pragma unroll
    for (int k = 1; k < MAXM - 1; ++k) {
        if (k <= m - 2) {
            Cx<R> a, b, c;
            coef(s + k, a, b, c);
            const Cx<R> denom = (k == 1) ? b : b - a * cprev;
            const Cx<R> inv = crecip(denom);
            const Cx<R> cp = c * inv;
            const Cx<R> yk = rhs(s + k);
            const Cx<R> da = (k == 1) ? yk * inv : (yk - a * daprev) * inv;
            const Cx<R> db = (k == 1) ? -(a * inv) : -((a * dbprev) * inv);
            glast = -(c * inv);
            al[k] = da;
            be[k] = db;
            // c' until the backward pass; on the last interior row gamma itself
            ga[k] = (k == m - 2) ? -(c * inv) : cp;
            cprev = cp;
            daprev = da;
            dbprev = db;
        }
    }
    // backward pass: alpha, beta, gamma
#pragma unroll
    for (int k = MAXM - 2; k >= 1; --k) {
        if (k < m - 2) {
            const Cx<R> cp = ga[k];
            al[k] = al[k] - cp * al[k + 1];
            be[k] = be[k] - cp * be[k + 1];
            ga[k] = -(cp * ga[k + 1]);
        }
    }
    // the chunk's first and last rows with the interior substituted
    Cx<R> aS, bS, cS, aE, bE, cE;
    coef(s, aS, bS, cS);
    coef(s + m - 1, aE, bE, cE);
    // alpha, beta, gamma of the last interior row are its forward-pass values
    const Cx<R> all = daprev, bel = dbprev, gal = glast;
    Cx<R> BS, CS, DS, AE, BE, DE;
    if (m >= 3) {
        BS = bS + cS * be[1];
        CS = cS * ga[1];
        DS = y0 - cS * al[1];
        AE = aE * bel;
        BE = bE + aE * gal;
        DE = yl - aE * all;
    } else {
        BS = bS;
        CS = cS;
        DS = y0;
        AE = aE;
        BE = bE;
        DE = yl;
    }
    const Cx<R> iS = crecip(BS), iE = crecip(BE);
    rowS.a = aS * iS;
    rowS.c = CS * iS;
    rowS.d = DS * iS;
    rowE.a = AE * iE;
    rowE.c = cE * iE;
    rowE.d = DE * iE;
}

// Phase 4: deliver x for the chunk given its end-point values.
template <typename R, int MAXM, class Out>
__device__ __forceinline__ void chunk_expand(int64_t s, int m, const Cx<R> (&al)[MAXM],
                                             const Cx<R> (&be)[MAXM], const Cx<R> (&ga)[MAXM],
                                             Cx<R> xs, Cx<R> xe, const Out& out) {
    out(s, xs);
#pragma unroll
    for (int k = 1; k < MAXM - 1; ++k)
        if (k <= m - 2) out(s + k, al[k] + be[k] * xs + ga[k] * xe);
    out(s + m - 1, xe);
}

// Phase 3: PCR over N = 2T normalised rows; thread t owns rows 2t and 2t+1
// (in ``r``) and leaves with their solution in r[q].d.  ``red`` is shared
// memory of pcr_smem_bytes<R>(T).  Must be called by all threads of the CTA.
template <typename R>
__device__ __forceinline__ void pcr_solve(int T, int t, bool active, Cx<R>* red, RedRow<R> (&r)[2]) {
    const Cx<R> zero = {R(0), R(0)};
    const int N = 2 * T;
    Cx<R>* Abuf = red;
    Cx<R>* Cbuf = red + 2 * N;
    Cx<R>* Dbuf = red + 4 * N;
    if (active) {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            Abuf[2 * t + q] = r[q].a;
            Cbuf[2 * t + q] = r[q].c;
            Dbuf[2 * t + q] = r[q].d;
        }
    }
    __syncthreads();
    const int levels = pcr_levels(N);
    int p = 0;
    for (int lev = 0, sig = 1; lev < levels; ++lev, sig <<= 1) {
        if (active) {
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int k = 2 * t + q;
                Cx<R> am = zero, cm = zero, dm = zero, ap = zero, cpp = zero, dp = zero;
                if (k - sig >= 0) {
                    am = Abuf[p * N + k - sig];
                    cm = Cbuf[p * N + k - sig];
                    dm = Dbuf[p * N + k - sig];
                }
                if (k + sig < N) {
                    ap = Abuf[p * N + k + sig];
                    cpp = Cbuf[p * N + k + sig];
                    dp = Dbuf[p * N + k + sig];
                }
                const Cx<R> a = r[q].a, c = r[q].c, d = r[q].d;
                const Cx<R> nb = Cx<R>{R(1), R(0)} - cm * a - ap * c;
                const Cx<R> na = -(am * a);
                const Cx<R> nc = -(cpp * c);
                const Cx<R> nd = d - dm * a - dp * c;
                const Cx<R> inv = crecip(nb);
                r[q].a = na * inv;
                r[q].c = nc * inv;
                r[q].d = nd * inv;
            }
            const int w = (p ^ 1) * N;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                Abuf[w + 2 * t + q] = r[q].a;
                Cbuf[w + 2 * t + q] = r[q].c;
                Dbuf[w + 2 * t + q] = r[q].d;
            }
        }
        p ^= 1;
        __syncthreads();
    }
}

// Whole-line solve by T threads (requires 2T <= n <= T*MAXM).
template <typename R, int MAXM, class Coef, class Rhs, class Out>
__device__ __forceinline__ void block_line_solve(int n, int T, int t, bool active, Cx<R>* red,
                                                 const Coef& coef, const Rhs& rhs, const Out& out) {
    int64_t s = 0;
    int m = 0;
    Cx<R> al[MAXM], be[MAXM], ga[MAXM];
    RedRow<R> r[2];
    if (active) {
        chunk_bounds(n, T, t, s, m);
        chunk_eliminate<R, MAXM>(s, m, coef, rhs, al, be, ga, r[0], r[1]);
    }
    pcr_solve<R>(T, t, active, red, r);
    if (active) chunk_expand<R, MAXM>(s, m, al, be, ga, r[0].d, r[1].d, out);
}

}  // namespace ion
