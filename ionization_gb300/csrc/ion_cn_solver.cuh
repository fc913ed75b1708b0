// Crank-Nicolson line solver used by every mesh kernel.
//
// Every implicit half-step of the mesh path solves A x = y with
// A = 1 + i B, B = tau * H real and tridiagonal (H a discretised Hamiltonian
// restricted to one line).  The solve is done in increment form: with psi the
// line before the step,
//     A (x - psi) = -i (w (B psi) + X)          x = psi + Delta
// where w = 2 when the explicit half-step acts along the same line
// (Crank-Nicolson: x = A^-1 (2 - A) psi) and w = 1 with X = (tau H' psi) the
// explicit half-step along the other direction of an ADI pass.  Solving for
// the increment keeps the rounding of the solve relative to |Delta| instead of
// |psi|, which matters for the complex64 state.
//
// Parallel scheme (as in ion_solver.cuh): T threads, thread t owns the M rows
// [t M, t M + M) (M compile-time, the line padded to T M rows with decoupled
// rows B = 0, psi = 0), partition-method elimination of each chunk in
// registers, PCR on the 2T reduced unknowns in shared memory, expansion.
// psi sits in shared memory interleaved by chunk: row i at slot
// (i % M) T + i / M, so the chunk reads of consecutive threads fall on
// consecutive slots.
//
// Functors:  coef(i, bo, bd): bo = B[i][i+1] (0 on the last row and on
// padding), bd = B[i][i] (0 on padding);  extra(i): X_i;  out(i, delta).
#pragma once

#include "ion_solver.cuh"

namespace ion {

template <int M>
__host__ __device__ __forceinline__ int islot(int i, int T) {
    return (i % M) * T + i / M;
}

// Reciprocal of a pivot's squared modulus.  FP64: correctly rounded.  FP32:
// the hardware approximation (PTX rcp.approx.ftz.f32, within 1 ulp; the
// pivots are of order one, never subnormal): the FP32 elimination's own
// rounding is of the same order, and the complex64 forms that need more
// accuracy refine the solve.
__device__ __forceinline__ float rcp_pivot(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double rcp_pivot(double x) { return __drcp_rn(x); }

template <typename R>
__device__ __forceinline__ Cx<R> crecip_fast(Cx<R> z) {
    const R inv = rcp_pivot(z.re * z.re + z.im * z.im);
    return {z.re * inv, -z.im * inv};
}

// cp.async (LDGSTS) helpers: global -> shared copies that bypass registers,
// completed with commit/wait groups
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Coefficients of the M rows [s, s + M) of one chunk; a coefficient type with
// a faster whole-chunk load provides its own overload.
template <int M, class Coef, typename R>
__device__ __forceinline__ void load_chunk(const Coef& coef, int s, R (&bo)[M], R (&bd)[M]) {
#pragma unroll
    for (int k = 0; k < M; ++k) coef(s + k, bo[k], bd[k]);
}

// (B psi)_i = a0 psi_{i-1} + bd psi_i + bo psi_{i+1}; a coefficient type that
// can form it without cancellation provides its own overload.
template <class Coef, typename R>
__device__ __forceinline__ Cx<R> stencil_row(const Coef&, int, R a0, R bd, R bo, Cx<R> p0, Cx<R> p1, Cx<R> p2) {
    return Cx<R>{a0 * p0.re + bd * p1.re + bo * p2.re, a0 * p0.im + bd * p1.im + bo * p2.im};
}

struct NoExtra {
    template <typename R>
    __device__ __forceinline__ Cx<R> get(int) const {
        return Cx<R>{R(0), R(0)};
    }
};

// Rows next to a chunk that another thread owns.  LocalHalo: the line ends
// at the first and last thread of the CTA.  ClusterHalo (the long-line
// kernel) continues the line into the neighbouring CTAs of a cluster.
struct LocalHalo {
    __device__ __forceinline__ bool has_left(int t) const { return t > 0; }
    __device__ __forceinline__ bool has_right(int t, int T) const { return t + 1 < T; }
    template <typename R, int M, class P>
    __device__ __forceinline__ Cx<R> left(const P& psi, int T, int t) const {
        return psi[(M - 1) * T + t - 1];
    }
    template <typename R, class P>
    __device__ __forceinline__ Cx<R> right(const P& psi, int T, int t) const {
        return psi[t + 1];
    }
};

// The line a solve reads (``psi`` of the functions below: a pointer to the
// interleaved shared-memory line, or a view with operator[]): psi + d / 2
// formed as it is read (``on``), or psi itself.
template <typename R>
struct HalfStepView {
    const Cx<R>* psi;
    const Cx<R>* d;
    bool on;
    __device__ __forceinline__ Cx<R> operator[](int i) const {
        const Cx<R> p = psi[i];
        if (!on) return p;
        const Cx<R> v = d[i];
        return Cx<R>{p.re + R(0.5) * v.re, p.im + R(0.5) * v.im};
    }
};

template <typename R, int M, class Coef, class Extra, class Halo = LocalHalo, class PsiT = const Cx<R>*>
__device__ __forceinline__ void cn_chunk_eliminate(int T, int t, R w, const PsiT& psi, const Coef& coef,
                                                   const Extra& extra, Cx<R> (&al)[M], Cx<R> (&be)[M],
                                                   Cx<R> (&ga)[M], RedRow<R>& rowS, RedRow<R>& rowE,
                                                   const Halo& halo = Halo{}) {
    static_assert(M >= 3, "chunks need an interior");
    const Cx<R> zero = {R(0), R(0)};
    const int s = t * M;
    R bo[M], bd[M];
    load_chunk<M>(coef, s, bo, bd);
    R bom1 = R(0);
    const bool hl = halo.has_left(t);
    if (hl) {
        R d_;
        coef(s - 1, bom1, d_);
    }
    // psi of the chunk with one neighbour on each side
    const Cx<R> pm1 = hl ? halo.template left<R, M>(psi, T, t) : zero;
    const Cx<R> pM = halo.has_right(t, T) ? halo.template right<R>(psi, T, t) : zero;
    auto P = [&](int k) -> Cx<R> { return k < 0 ? pm1 : (k >= M ? pM : psi[k * T + t]); };
    auto ao = [&](int k) -> R { return k == 0 ? bom1 : bo[k - 1]; };
    // y_k = -i (w (B psi)_k + X_k)
    auto Y = [&](int k) -> Cx<R> {
        const Cx<R> p0 = P(k - 1), p1 = P(k), p2 = P(k + 1);
        Cx<R> v = stencil_row(coef, s + k, ao(k), bd[k], bo[k], p0, p1, p2);
        const Cx<R> X = extra.template get<R>(s + k);
        v = Cx<R>{w * v.re + X.re, w * v.im + X.im};
        return Cx<R>{v.im, -v.re};  // -i v
    };

    Cx<R> cprev = zero, daprev = zero, dbprev = zero, glast = zero;
#pragma unroll
    for (int k = 1; k < M - 1; ++k) {
        const Cx<R> b = {R(1), bd[k]};
        const R a = ao(k);  // A[k][k-1] = i a
        const Cx<R> denom = (k == 1) ? b : b - mul_ih(a, cprev);
        const Cx<R> inv = crecip_fast(denom);
        const Cx<R> cp = mul_ih(bo[k], inv);
        const Cx<R> yk = Y(k);
        const Cx<R> da = (k == 1) ? yk * inv : (yk - mul_ih(a, daprev)) * inv;
        const Cx<R> db = (k == 1) ? -mul_ih(a, inv) : -(mul_ih(a, dbprev) * inv);
        glast = -cp;
        al[k] = da;
        be[k] = db;
        ga[k] = (k == M - 2) ? glast : cp;
        cprev = cp;
        daprev = da;
        dbprev = db;
    }
#pragma unroll
    for (int k = M - 3; k >= 1; --k) {
        const Cx<R> cp = ga[k];
        al[k] = al[k] - cp * al[k + 1];
        be[k] = be[k] - cp * be[k + 1];
        ga[k] = -(cp * ga[k + 1]);
    }
    // reduced rows: first row (coupled to the previous chunk's last unknown)
    const Cx<R> b0 = {R(1), bd[0]};
    const Cx<R> BS = b0 + mul_ih(bo[0], be[1]);
    const Cx<R> CS = mul_ih(bo[0], ga[1]);
    const Cx<R> DS = Y(0) - mul_ih(bo[0], al[1]);
    // last row (coupled to the next chunk's first unknown)
    const R aE = bo[M - 2];
    const Cx<R> bE = {R(1), bd[M - 1]};
    const Cx<R> AE = mul_ih(aE, dbprev);
    const Cx<R> BE = bE + mul_ih(aE, glast);
    const Cx<R> DE = Y(M - 1) - mul_ih(aE, daprev);
    const Cx<R> iS = crecip_fast(BS), iE = crecip_fast(BE);
    rowS.a = mul_ih(bom1, iS);
    rowS.c = CS * iS;
    rowS.d = DS * iS;
    rowE.a = AE * iE;
    rowE.c = mul_ih(bo[M - 1], iE);
    rowE.d = DE * iE;
}

// |re| + |im| (an upper bound of |z|) and the coupling below which a
// normalised reduced row counts as decoupled: 2^-30 in FP32, 2^-60 in FP64
template <typename R>
__device__ __forceinline__ R cabs1(Cx<R> z) {
    return fabs(z.re) + fabs(z.im);
}
template <typename R> struct PcrTiny;
template <> struct PcrTiny<float> {
    static constexpr float value = 9.3132257e-10f;
};
template <> struct PcrTiny<double> {
    static constexpr double value = 8.673617379884035e-19;
};

// The reduced system of the 2T chunk-end unknowns, solved on T rows.
// Thread t holds two normalised rows: r[0] for the first unknown of its
// chunk, xs_t = d - a xe_{t-1} - c xe_t, and r[1] for the last one,
// a xs_t + xe_t + c xs_{t+1} = d.  Substituting the first-row equations of
// threads t and t+1 into r[1] leaves one tridiagonal row in xe per thread
// (one step of odd-even reduction); PCR solves those T rows (ceil(log2 T)
// levels of one row per thread), and xs_t follows from r[0].  One region of
// 3 T complex words of ``red`` (pcr_cn_smem_bytes<R>(T)) holds, in turn, the
// first rows, each level's rows and the solved xe: every exchange reads its
// neighbours, meets a barrier, then writes.  On return r[0].d = xs_t and
// r[1].d = xe_t.
template <typename R>
__host__ __device__ constexpr size_t pcr_cn_smem_bytes(int T) {
    return 3 * size_t(T) * sizeof(Cx<R>);
}

template <typename R>
__device__ __forceinline__ void pcr_solve_cn(int T, int t, bool active, Cx<R>* red, RedRow<R> (&r)[2],
                                             R tiny = PcrTiny<R>::value) {
    const Cx<R> zero = {R(0), R(0)}, one = {R(1), R(0)};
    Cx<R>* A = red;
    Cx<R>* C = red + T;
    Cx<R>* D = red + 2 * T;
    if (active) {
        A[t] = r[0].a;
        C[t] = r[0].c;
        D[t] = r[0].d;
    }
    __syncthreads();
    RedRow<R> e = {zero, zero, zero};
    if (active) {
        Cx<R> an = zero, cn = zero, dn = zero;  // the next thread's first row
        if (t + 1 < T) {
            an = A[t + 1];
            cn = C[t + 1];
            dn = D[t + 1];
        }
        const RedRow<R>& S = r[0];
        const RedRow<R>& E = r[1];
        const Cx<R> inv = crecip_fast(one - E.a * S.c - E.c * an);
        e.a = -(E.a * S.a) * inv;
        e.c = -(E.c * cn) * inv;
        e.d = (E.d - E.a * S.d - E.c * dn) * inv;
    }
    __syncthreads();  // every first row is read
    if (active) {
        A[t] = e.a;
        C[t] = e.c;
        D[t] = e.d;
    }
    // the rows may already be decoupled below ``tiny`` (see the loop's exit)
    const bool coupled0 = active && (cabs1(e.a) > tiny || cabs1(e.c) > tiny);
    const int levels = __syncthreads_or(coupled0) ? pcr_levels(T) : 0;
    for (int lev = 0, sig = 1; lev < levels; ++lev, sig <<= 1) {
        Cx<R> am = zero, cm = zero, dm = zero, ap = zero, cpp = zero, dp = zero;
        if (active) {
            if (t - sig >= 0) {
                am = A[t - sig];
                cm = C[t - sig];
                dm = D[t - sig];
            }
            if (t + sig < T) {
                ap = A[t + sig];
                cpp = C[t + sig];
                dp = D[t + sig];
            }
        }
        __syncthreads();  // every neighbour row of this level is read
        if (active) {
            const Cx<R> a = e.a, c = e.c, d = e.d;
            const Cx<R> inv = crecip_fast(one - cm * a - ap * c);
            e.a = -(am * a) * inv;
            e.c = -(cpp * c) * inv;
            e.d = (d - dm * a - dp * c) * inv;
            A[t] = e.a;
            C[t] = e.c;
            D[t] = e.d;
        }
        // Early exit: once every row's couplings are below PcrTiny the
        // rows are decoupled to the working precision and x = d.  The
        // inverse of 1 + i tau H decays geometrically along a line: with
        // |tau H_i,i+1| ~ 0.3 (the spherical-harmonic sweeps) by ~0.26 per
        // row, so two or three levels of chunks of 8 rows already reach
        // this; a slowly decaying line runs every level.
        const bool coupled = active && (cabs1(e.a) > tiny || cabs1(e.c) > tiny);
        if (!__syncthreads_or(coupled)) break;
    }
    // D holds every xe (the barrier above ends the last write)
    if (active) {
        const Cx<R> xem1 = t > 0 ? D[t - 1] : zero;
        r[0].d = r[0].d - r[0].a * xem1 - r[0].c * e.d;
        r[1].d = e.d;
    }
}

// All threads of the CTA call this (threads t >= T only meet the barriers).
// ``out(i, delta)`` is called for the T*M rows of the padded line.
// ``tiny``: the coupling below which the reduced system's rows count as
// decoupled (PcrTiny: to the working precision).
template <typename R, int M, class Coef, class Extra, class Out, class PsiT = const Cx<R>*>
__device__ __forceinline__ void block_cn_solve(int T, int t, R w, const PsiT& psi, Cx<R>* red, const Coef& coef,
                                               const Extra& extra, const Out& out, R tiny = PcrTiny<R>::value) {
    const bool active = t < T;
    Cx<R> al[M], be[M], ga[M];
    RedRow<R> r[2];
    if (active) cn_chunk_eliminate<R, M>(T, t, w, psi, coef, extra, al, be, ga, r[0], r[1]);
    pcr_solve_cn<R>(T, t, active, red, r, tiny);
    if (active) {
        const int s = t * M;
        const Cx<R> xs = r[0].d, xe = r[1].d;
        out(s, xs);
#pragma unroll
        for (int k = 1; k < M - 1; ++k) out(s + k, al[k] + be[k] * xs + ga[k] * xe);
        out(s + M - 1, xe);
    }
}

// ---------------------------------------------------------------------------
// Rotation coefficients cos(a) - 1 and sin(a).
// |a| <= 0.5: Maclaurin series of sin and cos, as polynomials in a^2 with
// the coefficients (-1)^k / n! evaluated by Horner's rule (one fma per
// term):
//   sin a = a + (a a^2) P(a^2),   cos a - 1 = a^2 Q(a^2),
// truncated where the next term is below 1e-10 of the result in FP32 and
// below 1e-19 in FP64: for |a| <= 1/16 (most angles of a step) after
// a^5 / a^6 in FP32 and a^9 / a^10 in FP64, else after a^9 / a^10 and
// a^19 / a^20.  Otherwise sincos() with cos(a) - 1 = -2 sin^2(a/2).  The
// branch depends on a alone, so every launch shape gives the same bits.
// Returning cos - 1 lets the rotation be applied in increment form.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void rot_coeffs(float a, float& cm1, float& s) {
    if (fabsf(a) <= 0.0625f) {
        const float a2 = a * a;
        const float p = fmaf(1.f / 120.f, a2, -1.f / 6.f);
        s = fmaf(a * a2, p, a);
        float q = fmaf(-1.f / 720.f, a2, 1.f / 24.f);
        q = fmaf(q, a2, -0.5f);
        cm1 = a2 * q;
    } else if (fabsf(a) <= 0.5f) {
        const float a2 = a * a;
        float p = 1.f / 362880.f;               // 1/9!
        p = fmaf(p, a2, -1.f / 5040.f);         // -1/7!
        p = fmaf(p, a2, 1.f / 120.f);           // 1/5!
        p = fmaf(p, a2, -1.f / 6.f);            // -1/3!
        s = fmaf(a * a2, p, a);
        float q = -1.f / 3628800.f;             // -1/10!
        q = fmaf(q, a2, 1.f / 40320.f);         // 1/8!
        q = fmaf(q, a2, -1.f / 720.f);          // -1/6!
        q = fmaf(q, a2, 1.f / 24.f);            // 1/4!
        q = fmaf(q, a2, -0.5f);                 // -1/2!
        cm1 = a2 * q;
    } else {
        float c;
        sincosf(a, &s, &c);
        const float h = sinf(0.5f * a);
        cm1 = -2.f * h * h;
    }
}

__device__ __forceinline__ void rot_coeffs(double a, double& cm1, double& s) {
    if (fabs(a) <= 0.0625) {
        const double a2 = a * a;
        double p = 1.0 / 362880.0;        // 1/9!
        p = fma(p, a2, -1.0 / 5040.0);    // -1/7!
        p = fma(p, a2, 1.0 / 120.0);      // 1/5!
        p = fma(p, a2, -1.0 / 6.0);       // -1/3!
        s = fma(a * a2, p, a);
        double q = -1.0 / 3628800.0;      // -1/10!
        q = fma(q, a2, 1.0 / 40320.0);    // 1/8!
        q = fma(q, a2, -1.0 / 720.0);     // -1/6!
        q = fma(q, a2, 1.0 / 24.0);       // 1/4!
        q = fma(q, a2, -0.5);             // -1/2!
        cm1 = a2 * q;
    } else if (fabs(a) <= 0.5) {
        const double a2 = a * a;
        // 1/n! for odd n = 19 .. 3 and even n = 20 .. 2, alternating in sign
        double p = -1.0 / 121645100408832000.0;  // -1/19!
        p = fma(p, a2, 1.0 / 355687428096000.0);  // 1/17!
        p = fma(p, a2, -1.0 / 1307674368000.0);   // -1/15!
        p = fma(p, a2, 1.0 / 6227020800.0);       // 1/13!
        p = fma(p, a2, -1.0 / 39916800.0);        // -1/11!
        p = fma(p, a2, 1.0 / 362880.0);           // 1/9!
        p = fma(p, a2, -1.0 / 5040.0);            // -1/7!
        p = fma(p, a2, 1.0 / 120.0);              // 1/5!
        p = fma(p, a2, -1.0 / 6.0);               // -1/3!
        s = fma(a * a2, p, a);
        double q = 1.0 / 2432902008176640000.0;   // 1/20!
        q = fma(q, a2, -1.0 / 6402373705728000.0);  // -1/18!
        q = fma(q, a2, 1.0 / 20922789888000.0);     // 1/16!
        q = fma(q, a2, -1.0 / 87178291200.0);       // -1/14!
        q = fma(q, a2, 1.0 / 479001600.0);          // 1/12!
        q = fma(q, a2, -1.0 / 3628800.0);           // -1/10!
        q = fma(q, a2, 1.0 / 40320.0);              // 1/8!
        q = fma(q, a2, -1.0 / 720.0);               // -1/6!
        q = fma(q, a2, 1.0 / 24.0);                 // 1/4!
        q = fma(q, a2, -0.5);                       // -1/2!
        cm1 = a2 * q;
    } else {
        double c;
        sincos(a, &s, &c);
        const double h = sin(0.5 * a);
        cm1 = -2.0 * h * h;
    }
}

}  // namespace ion
