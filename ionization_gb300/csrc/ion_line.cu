// Line mesh, length gauge: LineMesh (ionization/mesh/meshes.py:263-341) with
// LineLengthGaugeOperators (ionization/mesh/mesh_operators.py:304-341) under
// AlternatingDirectionImplicit or SplitInteractionOperator
// (ionization/mesh/evolution_methods.py:46-123), then the mask
// (meshes.py:256-257).
//
// One CTA owns one simulation for a whole step: psi is staged in shared
// memory (interleaved by solver chunk), the Crank-Nicolson step is solved in
// increment form by the block partition + PCR solver (ion_cn_solver.cuh),
// the split-operator phase factors and the mask are applied on the way in and
// out, and at data times the norm / inner products are reduced from shared
// memory before psi is stored.
#include <cooperative_groups.h>

#include <type_traits>

#include "ion_common.cuh"
#include "ion_cn_solver.cuh"

namespace cg = cooperative_groups;

namespace ion {

template <typename R> struct LineCfg;
template <> struct LineCfg<double> {
    static constexpr int M = 8;
    static constexpr int MAX_T = 512;
};
template <> struct LineCfg<float> {
    static constexpr int M = 16;
    static constexpr int MAX_T = 512;
};

__host__ __device__ inline int line_threads(int n, int m) { return (n + m - 1) / m; }

__device__ __forceinline__ bool line_is_data(int64_t t, int64_t tf, int64_t every) {
    return t == 0 || t == tf || (every >= 1 && t % every == 0);
}
__device__ __forceinline__ int64_t line_slot(int64_t t, int64_t tf, int64_t every) {
    if (every >= 1) return (t % every == 0) ? t / every : tf / every + 1;
    return t == 0 ? 0 : 1;
}

template <typename R> struct LineTab;
template <> struct LineTab<double> {
    const double *hd, *hoff, *zq, *mask;
    __device__ static LineTab make(const ion_line_sim& S) { return {S.hd, S.hoff, S.zq, S.mask}; }
};
template <> struct LineTab<float> {
    const float *hd, *hoff, *zq, *mask;
    __device__ static LineTab make(const ion_line_sim& S) { return {S.hd32, S.hoff32, S.zq32, S.mask32}; }
};

// tau-scaled H: H0 + diag(zq E) for ADI, H0 for the split operator
template <typename R>
struct LineCnCoef {
    LineTab<R> tb;
    R tau, efield;
    bool with_field;
    int n;
    __device__ __forceinline__ void operator()(int i, R& bo, R& bd) const {
        if (i >= n) {
            bo = R(0);
            bd = R(0);
            return;
        }
        const R h = with_field ? fma(tb.zq[i], efield, tb.hd[i]) : tb.hd[i];
        bd = tau * h;
        bo = (i < n - 1) ? tau * tb.hoff[i] : R(0);
    }
};

template <typename R, int M>
struct LineAddOut {
    Cx<R>* line;
    int T;
    __device__ __forceinline__ void operator()(int i, Cx<R> d) const {
        Cx<R>* p = line + islot<M>(i, T);
        *p = *p + d;
    }
};

// x * exp(-i theta) in increment form
template <typename R>
__device__ __forceinline__ Cx<R> phase(Cx<R> x, R theta) {
    R cm1, s;
    rot_coeffs(theta, cm1, s);
    return Cx<R>{x.re + (cm1 * x.re + s * x.im), x.im + (cm1 * x.im - s * x.re)};
}

__device__ __forceinline__ double block_sum_l(double v, double* scratch) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) scratch[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        for (int i = 0; i < nw; ++i) r += scratch[i];
    }
    return r;
}

// norm and inner products of the line held in shared memory (FP64).  The
// first ``stride`` threads (a count fixed by the simulation alone) take rows
// i = thread + k stride, so the sums do not depend on the CTA size of the
// launch, i.e. on the other simulations of a plan.
template <typename R, int M>
__device__ void line_reduce(const ion_line_sim& S, const Cx<R>* line, int T, int stride, int64_t t,
                            double* scratch) {
    const int n = S.n;
    const int64_t slot = line_slot(t, S.t_final, S.store_every);
    const int i0 = int(threadIdx.x) < stride ? int(threadIdx.x) : n;
    double acc = 0.0;
    for (int i = i0; i < n; i += stride) {
        const Cx<R> x = line[islot<M>(i, T)];
        acc += double(x.re) * double(x.re) + double(x.im) * double(x.im);
    }
    const double nrm = block_sum_l(acc, scratch);
    if (threadIdx.x == 0) S.out_norm[slot] = nrm * S.weight;
    for (int s = 0; s < S.n_states; ++s) {
        const double* sg = S.state_g + int64_t(s) * n * 2;
        double re = 0.0, im = 0.0;
        for (int i = i0; i < n; i += stride) {
            const Cx<R> x = line[islot<M>(i, T)];
            const double ar = sg[2 * i], ai = -sg[2 * i + 1];
            re += ar * double(x.re) - ai * double(x.im);
            im += ar * double(x.im) + ai * double(x.re);
        }
        const double tr = block_sum_l(re, scratch);
        const double ti = block_sum_l(im, scratch);
        if (threadIdx.x == 0) {
            S.out_ip[(slot * S.n_states + s) * 2] = tr * S.weight;
            S.out_ip[(slot * S.n_states + s) * 2 + 1] = ti * S.weight;
        }
    }
}

// words of the region after the line: the reduced system of a
// Crank-Nicolson line, or (a plan with Fourier split-step lines, ION_LINE_HAS_FFT)
// the cached phase factors of a Fourier line, whichever is larger
template <typename R>
__host__ __device__ inline size_t line_red_words(int threads, int M, bool fft) {
    const size_t cn = pcr_smem_bytes<R>(threads) / sizeof(Cx<R>);
    const size_t ft = fft ? 2 * size_t(threads) * M : 0;
    return cn > ft ? cn : ft;
}
template <typename R>
__host__ __device__ inline size_t line_smem(int threads, int M, bool fft = false) {
    return (size_t(threads) * M + line_red_words<R>(threads, M, fft)) * sizeof(Cx<R>) + 32 * sizeof(double);
}

// ---------------------------------------------------------------------------
// Fourier split-step (ION_LINE_FFT; the reference evolves lines only with
// Crank-Nicolson):
//   psi <- mask * P F^-1 K F P psi,
//   P = exp(-i tau (V + zq E(t_{n+1}))),  K = exp(-i 2 tau E_kin(k)) / n,
// periodic in z.  F is an in-place radix-4 decimation-in-frequency FFT of the
// line held in shared memory (n = 2^k, a final radix-2 stage when k is odd).
// Every radix-4 butterfly stores its outputs in the order of two radix-2
// stages, so the spectrum comes out in bit-reversed order; K is tabulated in
// that order and the inverse applies the exact inverse of each forward
// butterfly in reverse order, which gives back natural order (times n, folded
// into K).  No reordering pass is needed.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ Cx<R> ldg_cx(const Cx<R>* p) {
    const typename Vec2<R>::type v = __ldg(reinterpret_cast<const typename Vec2<R>::type*>(p));
    return {v.x, v.y};
}
template <typename R>
__device__ __forceinline__ Cx<R> mul_conj(Cx<R> a, Cx<R> w) {  // a * conj(w)
    return {a.re * w.re + a.im * w.im, a.im * w.re - a.re * w.im};
}
template <typename R>
__device__ __forceinline__ Cx<R> mul_minus_i(Cx<R> a) { return {a.im, -a.re}; }
template <typename R>
__device__ __forceinline__ Cx<R> mul_plus_i(Cx<R> a) { return {-a.im, a.re}; }

// forward radix-4 stage over blocks of 4q points, q = 2^lq; tw[m] = exp(-2 pi i m / n)
template <typename R>
__device__ __forceinline__ void fft_dif4(Cx<R>* x, int n, int lq, const Cx<R>* __restrict__ tw) {
    const int q = 1 << lq;
    const int s = n >> (lq + 2);  // w_{4q}^j = tw[j s]
    for (int b = threadIdx.x; b < (n >> 2); b += blockDim.x) {
        const int k = b & (q - 1);
        const int i0 = ((b >> lq) << (lq + 2)) + k;
        const Cx<R> a0 = x[i0], a1 = x[i0 + q], a2 = x[i0 + 2 * q], a3 = x[i0 + 3 * q];
        const Cx<R> t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = mul_minus_i(a1 - a3);
        x[i0] = t0 + t2;
        x[i0 + q] = (t0 - t2) * ldg_cx(tw + 2 * k * s);
        x[i0 + 2 * q] = (t1 + t3) * ldg_cx(tw + k * s);
        x[i0 + 3 * q] = (t1 - t3) * ldg_cx(tw + 3 * k * s);
    }
}

// inverse of fft_dif4 (times 4)
template <typename R>
__device__ __forceinline__ void fft_dif4_inverse(Cx<R>* x, int n, int lq, const Cx<R>* __restrict__ tw) {
    const int q = 1 << lq;
    const int s = n >> (lq + 2);
    for (int b = threadIdx.x; b < (n >> 2); b += blockDim.x) {
        const int k = b & (q - 1);
        const int i0 = ((b >> lq) << (lq + 2)) + k;
        const Cx<R> y0 = x[i0];
        const Cx<R> u2 = mul_conj(x[i0 + q], ldg_cx(tw + 2 * k * s));
        const Cx<R> u1 = mul_conj(x[i0 + 2 * q], ldg_cx(tw + k * s));
        const Cx<R> u3 = mul_conj(x[i0 + 3 * q], ldg_cx(tw + 3 * k * s));
        const Cx<R> t0 = y0 + u2, t2 = y0 - u2, t1 = u1 + u3, t3 = mul_plus_i(u1 - u3);
        x[i0] = t0 + t1;
        x[i0 + 2 * q] = t0 - t1;
        x[i0 + q] = t2 + t3;
        x[i0 + 3 * q] = t2 - t3;
    }
}

// radix-2 stage over blocks of 2 points (its own inverse, times 2)
template <typename R>
__device__ __forceinline__ void fft_pairs(Cx<R>* x, int n) {
    for (int j = threadIdx.x; j < (n >> 1); j += blockDim.x) {
        const Cx<R> a = x[2 * j], b = x[2 * j + 1];
        x[2 * j] = a + b;
        x[2 * j + 1] = a - b;
    }
}

template <typename R> struct FftTab;
template <> struct FftTab<double> {
    const double *v, *zq, *mask;
    __device__ static FftTab make(const ion_line_sim& S) { return {S.vstat, S.zq, S.mask}; }
};
template <> struct FftTab<float> {
    const float *v, *zq, *mask;
    __device__ static FftTab make(const ion_line_sim& S) { return {S.vstat32, S.zq32, S.mask32}; }
};

// the kinetic phase angle 2 tau E_kin is formed in FP64; the FP32 path reduces
// it to [-pi, pi] first so that its rounding is relative to the reduced angle
template <typename R> __device__ __forceinline__ R kinetic_angle(double a);
template <> __device__ __forceinline__ double kinetic_angle<double>(double a) { return a; }
template <> __device__ __forceinline__ float kinetic_angle<float>(double a) {
    const double turns = rint(a * 0.15915494309189535);  // a / (2 pi), to the nearest integer
    return float(fma(-turns, 6.283185307179586, a));
}

// x * exp(-i theta) from theta's rotation coefficients c = (cos - 1, sin),
// as phase() forms it
template <typename R>
__device__ __forceinline__ Cx<R> apply_phase(Cx<R> x, Cx<R> c) {
    return Cx<R>{x.re + (c.re * x.re + c.im * x.im), x.im + (c.re * x.im - c.im * x.re)};
}

// One step of a Fourier line held in x.  pc[n], kc[n]: the step's potential
// phase and the kinetic phase (cos - 1, sin) per point, cached in shared
// memory: the potential phase is applied twice per step from one evaluation,
// and the kinetic phase, which depends on tau alone, is evaluated again only
// when tau changes (ktau: the tau kc holds, the same in every thread).  The
// arithmetic is that of evaluating every phase where it is applied.
template <typename R>
__device__ void line_fft_step(ion_line_sim& S, int64_t t, Cx<R>* x, int stride, double* scratch, Cx<R>* pc,
                              Cx<R>* kc, double& ktau) {
    const int n = S.n;
    const int lg = 31 - __clz(n);
    const FftTab<R> tb = FftTab<R>::make(S);
    const Cx<R>* tw = static_cast<const Cx<R>*>(S.twiddle);
    Cx<R>* g = static_cast<Cx<R>*>(S.g);
    const double tau = S.tau[t + 1];
    const R taur = R(tau), ef = R(S.efield[t + 1]);

    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Cx<R> c;
        rot_coeffs(taur * (tb.v[i] + tb.zq[i] * ef), c.re, c.im);
        pc[i] = c;
        x[i] = apply_phase(ld(g + i), c);
    }
    __syncthreads();
    for (int lq = lg - 2; lq >= 0; lq -= 2) {
        fft_dif4(x, n, lq, tw);
        __syncthreads();
    }
    if (lg & 1) {
        fft_pairs(x, n);
        __syncthreads();
    }
    const R inv_n = R(1) / R(n);  // exact: n is a power of two
    const bool fresh = tau != ktau;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        if (fresh) {
            Cx<R> c;
            rot_coeffs(kinetic_angle<R>(2.0 * tau * S.kin[i]), c.re, c.im);
            kc[i] = c;
        }
        x[i] = scale(apply_phase(x[i], kc[i]), inv_n);
    }
    ktau = tau;
    __syncthreads();
    if (lg & 1) {
        fft_pairs(x, n);
        __syncthreads();
    }
    for (int lq = lg & 1; lq <= lg - 2; lq += 2) {
        fft_dif4_inverse(x, n, lq, tw);
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Cx<R> y = apply_phase(x[i], pc[i]);
        if (tb.mask) y = Cx<R>{y.re * tb.mask[i], y.im * tb.mask[i]};
        x[i] = y;
        st(g + i, y);
    }
    __syncthreads();
    if (line_is_data(t + 1, S.t_final, S.store_every)) line_reduce<R, 1>(S, x, n, stride, t + 1, scratch);
    __syncthreads();
}

// The velocity gauge's split operator on a line held in shared memory: the
// pairs (i, i+1) for i = parity, parity + 2, ... turn by [[cos, sin],
// [-sin, cos]] (cm1 = cos - 1 for the increment form)
template <typename R, int M>
__device__ __forceinline__ void line_pair_rotations(Cx<R>* line, int n, int T, int parity, R cm1, R s) {
    for (int i = parity + 2 * int(threadIdx.x); i + 1 < n; i += 2 * int(blockDim.x)) {
        Cx<R>* p0 = line + islot<M>(i, T);
        Cx<R>* p1 = line + islot<M>(i + 1, T);
        const Cx<R> x0 = *p0, x1 = *p1;
        *p0 = Cx<R>{x0.re + (cm1 * x0.re + s * x1.re), x0.im + (cm1 * x0.im + s * x1.im)};
        *p1 = Cx<R>{x1.re + (cm1 * x1.re - s * x0.re), x1.im + (cm1 * x1.im - s * x0.im)};
    }
    __syncthreads();
}

// mode 0: up to n_steps steps (each followed by the reductions at a data
// time), ending at t_final; mode 1: the reductions at t only
template <typename R, int M>
__global__ void __launch_bounds__(512) line_step_kernel(ion_line_plan plan, int mode, int n_steps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ion_line_sim& S = plan.sims[blockIdx.x];
    const int64_t t0 = S.t, tf = S.t_final;
    const int n = S.n;
    const int T = line_threads(n, M);
    const int npad = T * M;
    Cx<R>* line = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* red = line + plan.threads * M;
    const bool fft_plan = (plan.flags & ION_LINE_HAS_FFT) != 0;
    double* scratch = reinterpret_cast<double*>(red + line_red_words<R>(plan.threads, M, fft_plan));
    Cx<R>* g = static_cast<Cx<R>*>(S.g);
    const Cx<R> zero = {R(0), R(0)};
    if (n < 2 || n > plan.max_n) return;  // the plan's shared memory is sized for max_n
    // a Fourier line needs the phase caches (ION_LINE_HAS_FFT): without them
    // it is left untouched, like a line of another plan
    if (S.method == ION_LINE_FFT && !fft_plan) return;
    double ktau = -1.0;  // no kinetic phase cached yet (tau > 0)

    if (mode == 1) {
        if (!line_is_data(t0, tf, S.store_every)) return;
        for (int i = threadIdx.x; i < n; i += blockDim.x) line[islot<M>(i, T)] = ld(g + i);
        __syncthreads();
        line_reduce<R, M>(S, line, T, T, t0, scratch);
        return;
    }
    const int64_t tend = tf - t0 > n_steps ? t0 + n_steps : tf;
    if (t0 >= tend) return;
    for (int64_t t = t0; t < tend; ++t) {  // each step ends with a CTA barrier
    if (S.method == ION_LINE_FFT) {
        line_fft_step<R>(S, t, line, T, scratch, red, red + plan.threads * M, ktau);
        continue;
    }
    const LineTab<R> tb = LineTab<R>::make(S);
    const R tau = R(S.tau[t + 1]);
    const R ef = R(S.efield[t + 1]);
    const bool vel = S.gauge == ION_GAUGE_VELOCITY;  // ef is then A(t)
    const bool split = S.method == ION_LINE_SPLIT && !vel;
    R vcm1 = R(0), vs = R(0);
    if (vel) rot_coeffs(R(S.tau[t + 1] * S.efield[t + 1] * S.vcoef), vcm1, vs);

#pragma unroll
    for (int k = 0; k < M; ++k) {  // npad <= blockDim * M: loads issue together
        const int i = threadIdx.x + k * blockDim.x;
        if (i >= npad) continue;
        Cx<R> x = zero;
        if (i < n) {
            x = ld(g + i);
            if (split) x = phase(x, (tb.zq[i] * ef) * tau);  // exp(-i tau V_int)
        }
        line[islot<M>(i, T)] = x;
    }
    __syncthreads();
    if (vel) {
        line_pair_rotations<R, M>(line, n, T, 0, vcm1, vs);
        line_pair_rotations<R, M>(line, n, T, 1, vcm1, vs);
    }
    const LineCnCoef<R> coef{tb, tau, ef, S.method == ION_LINE_ADI, n};
    block_cn_solve<R, M>(T, threadIdx.x, R(2), line, red, coef, NoExtra{}, LineAddOut<R, M>{line, T});
    __syncthreads();
    if (vel) {
        line_pair_rotations<R, M>(line, n, T, 1, vcm1, vs);
        line_pair_rotations<R, M>(line, n, T, 0, vcm1, vs);
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Cx<R>* p = line + islot<M>(i, T);
        Cx<R> x = *p;
        if (split) x = phase(x, (tb.zq[i] * ef) * tau);
        if (tb.mask) x = Cx<R>{x.re * tb.mask[i], x.im * tb.mask[i]};
        *p = x;
        st(g + i, x);
    }
    __syncthreads();
    if (line_is_data(t + 1, tf, S.store_every)) line_reduce<R, M>(S, line, T, T, t + 1, scratch);
    __syncthreads();
    }
    if (threadIdx.x == 0) S.t = tend;  // every thread read S.t before the first barrier
}

// ---------------------------------------------------------------------------
// Lines longer than one CTA holds: one thread-block cluster of C CTAs per
// simulation.  CTA r holds rows [r T M, (r+1) T M) of the line in its shared
// memory, with the same per-thread chunks as the one-CTA kernel.  The chunk
// halos at a segment edge are read from the neighbouring CTA's shared memory
// (DSMEM), and the PCR of the 2 T C reduced rows runs across the cluster, the
// rows of other CTAs read through DSMEM, one cluster barrier per level.  Data
// reductions are summed per CTA, gathered on rank 0 and added in rank order.
// Every CTA of a cluster works on the same simulation, so every early return
// is taken by the whole cluster.
// ---------------------------------------------------------------------------
template <typename R>
struct ClusterHalo {
    const Cx<R>* prev;  // line of the previous CTA (DSMEM), nullptr on rank 0
    const Cx<R>* next;  // line of the next CTA, nullptr on the last rank
    __device__ __forceinline__ bool has_left(int t) const { return t > 0 || prev != nullptr; }
    __device__ __forceinline__ bool has_right(int t, int T) const { return t + 1 < T || next != nullptr; }
    template <typename RR, int M>
    __device__ __forceinline__ Cx<RR> left(const Cx<RR>* psi, int T, int t) const {
        return t > 0 ? psi[(M - 1) * T + t - 1] : reinterpret_cast<const Cx<RR>*>(prev)[(M - 1) * T + T - 1];
    }
    template <typename RR>
    __device__ __forceinline__ Cx<RR> right(const Cx<RR>* psi, int T, int t) const {
        return t + 1 < T ? psi[t + 1] : reinterpret_cast<const Cx<RR>*>(next)[0];
    }
};

template <typename R>
struct OffsetCoef {
    LineCnCoef<R> c;
    int off;
    __device__ __forceinline__ void operator()(int i, R& bo, R& bd) const { c(off + i, bo, bd); }
};

// The reduced system of a line split over the C CTAs of a cluster, in the
// form pcr_solve_cn uses for one CTA: thread t of CTA r holds the two rows of
// its chunk ends; one step of odd-even reduction leaves one row per thread
// (the first row of thread t + 1 comes from the next CTA for t = T - 1), PCR
// solves the T C rows of the cluster (global row r T + t; rows of other CTAs
// through distributed shared memory, one cluster barrier per level), and the
// chunk-start unknowns follow from the left neighbour's chunk-end unknown.
// Uses 9 T complex words of ``red``.  The last read of another CTA's ``red``
// comes after the last barrier here: the caller holds a cluster barrier
// before ``red`` is written again or the CTA exits.  On return
// r[0].d = xs_t and r[1].d = xe_t.
template <typename R>
__device__ __forceinline__ void pcr_solve_cluster(int T, int t, bool active, Cx<R>* red, RedRow<R> (&r)[2],
                                                  int rank, int C) {
    cg::cluster_group cl = cg::this_cluster();
    const Cx<R> zero = {R(0), R(0)}, one = {R(1), R(0)};
    Cx<R>* Sa = red;
    Cx<R>* Sc = red + T;
    Cx<R>* Sd = red + 2 * T;
    Cx<R>* Ab = red + 3 * T;  // double-buffered [2][T]
    Cx<R>* Cb = red + 5 * T;
    Cx<R>* Db = red + 7 * T;
    if (active) {
        Sa[t] = r[0].a;
        Sc[t] = r[0].c;
        Sd[t] = r[0].d;
    }
    cl.sync();
    RedRow<R> e = {zero, zero, zero};
    if (active) {
        Cx<R> an = zero, cn = zero, dn = zero;  // the next thread's first row
        if (t + 1 < T) {
            an = Sa[t + 1];
            cn = Sc[t + 1];
            dn = Sd[t + 1];
        } else if (rank + 1 < C) {
            an = cl.map_shared_rank(Sa, rank + 1)[0];
            cn = cl.map_shared_rank(Sc, rank + 1)[0];
            dn = cl.map_shared_rank(Sd, rank + 1)[0];
        }
        const RedRow<R>& S0 = r[0];
        const RedRow<R>& E = r[1];
        const Cx<R> inv = crecip_fast(one - E.a * S0.c - E.c * an);
        e.a = -(E.a * S0.a) * inv;
        e.c = -(E.c * cn) * inv;
        e.d = (E.d - E.a * S0.d - E.c * dn) * inv;
        Ab[t] = e.a;
        Cb[t] = e.c;
        Db[t] = e.d;
    }
    cl.sync();
    const int NT = T * C;
    const int levels = pcr_levels(NT);
    // owner CTA of global row k: floor(k / T) as (k + 1/2) * (1 / T) in FP32,
    // exact here: the quotient stays >= 1/(2T) >= 2^-10 from an integer while
    // k < 2^13 keeps the rounding below 2^-20
    const float invT = 1.f / float(T);
    // row k at level buffer ``base``: local rows through the shared window,
    // other CTAs' rows through distributed shared memory
    auto fetch = [&](int k, int base, Cx<R>& a_, Cx<R>& c_, Cx<R>& d_) {
        const int o = int((float(k) + 0.5f) * invT);
        const int sl = base + (k - o * T);
        if (o == rank) {
            a_ = Ab[sl];
            c_ = Cb[sl];
            d_ = Db[sl];
        } else {
            a_ = cl.map_shared_rank(Ab, o)[sl];
            c_ = cl.map_shared_rank(Cb, o)[sl];
            d_ = cl.map_shared_rank(Db, o)[sl];
        }
    };
    const int k0 = rank * T + t;
    int p = 0;
    for (int lev = 0, sig = 1; lev < levels; ++lev, sig <<= 1) {
        if (active) {
            const int base = p * T;
            Cx<R> am = zero, cm = zero, dm = zero, ap = zero, cpp = zero, dp = zero;
            if (k0 - sig >= 0) fetch(k0 - sig, base, am, cm, dm);
            if (k0 + sig < NT) fetch(k0 + sig, base, ap, cpp, dp);
            const Cx<R> a = e.a, c = e.c, d = e.d;
            const Cx<R> inv = crecip_fast(one - cm * a - ap * c);
            e.a = -(am * a) * inv;
            e.c = -(cpp * c) * inv;
            e.d = (d - dm * a - dp * c) * inv;
            const int wb = (p ^ 1) * T;
            Ab[wb + t] = e.a;
            Cb[wb + t] = e.c;
            Db[wb + t] = e.d;
        }
        p ^= 1;
        cl.sync();
    }
    // Db[p T + .] holds every thread's chunk-end unknown
    if (active) {
        Cx<R> xem1 = zero;
        if (t > 0)
            xem1 = Db[p * T + t - 1];
        else if (rank > 0)
            xem1 = cl.map_shared_rank(Db, rank - 1)[p * T + T - 1];
        r[0].d = r[0].d - r[0].a * xem1 - r[0].c * e.d;
        r[1].d = e.d;
    }
}

// sum of one or two doubles (valid in thread 0 of each CTA) over the cluster,
// added in rank order on rank 0; ``part`` is 32 doubles of shared memory,
// double-buffered by ``round`` so one cluster barrier per round suffices
__device__ __forceinline__ void cluster_sum2(double& a, double& b, double* part, int round, int rank, int C) {
    cg::cluster_group cl = cg::this_cluster();
    double* buf = part + (round & 1) * 16;
    if (threadIdx.x == 0) {
        double* dst = cl.map_shared_rank(buf, 0);
        dst[2 * rank] = a;
        dst[2 * rank + 1] = b;
    }
    cl.sync();
    if (rank == 0 && threadIdx.x == 0) {
        a = 0.0;
        b = 0.0;
        for (int k = 0; k < C; ++k) {
            a += buf[2 * k];
            b += buf[2 * k + 1];
        }
    }
}

template <typename R, int M>
__device__ void line_reduce_cluster(const ion_line_sim& S, const Cx<R>* line, int T, int off, int64_t t,
                                    double* scratch, double* part, int rank, int C) {
    const int n = S.n;
    const int L = T * M;
    const int64_t slot = line_slot(t, S.t_final, S.store_every);
    const int i0 = int(threadIdx.x) < T ? int(threadIdx.x) : L;  // see line_reduce
    double acc = 0.0;
    for (int i = i0; i < L && off + i < n; i += T) {
        const Cx<R> x = line[islot<M>(i, T)];
        acc += double(x.re) * double(x.re) + double(x.im) * double(x.im);
    }
    double nrm = block_sum_l(acc, scratch), unused = 0.0;
    cluster_sum2(nrm, unused, part, 0, rank, C);
    if (rank == 0 && threadIdx.x == 0) S.out_norm[slot] = nrm * S.weight;
    for (int s = 0; s < S.n_states; ++s) {
        const double* sg = S.state_g + int64_t(s) * n * 2;
        double re = 0.0, im = 0.0;
        for (int i = i0; i < L && off + i < n; i += T) {
            const Cx<R> x = line[islot<M>(i, T)];
            const double ar = sg[2 * (off + i)], ai = -sg[2 * (off + i) + 1];
            re += ar * double(x.re) - ai * double(x.im);
            im += ar * double(x.im) + ai * double(x.re);
        }
        double tr = block_sum_l(re, scratch);
        double ti = block_sum_l(im, scratch);
        cluster_sum2(tr, ti, part, s + 1, rank, C);
        if (rank == 0 && threadIdx.x == 0) {
            S.out_ip[(slot * S.n_states + s) * 2] = tr * S.weight;
            S.out_ip[(slot * S.n_states + s) * 2 + 1] = ti * S.weight;
        }
    }
}

template <typename R>
__host__ __device__ inline size_t line_cluster_smem(int threads, int M) {
    return line_smem<R>(threads, M) + 32 * sizeof(double);
}

// Crank-Nicolson methods only (ION_LINE_ADI / ION_LINE_SPLIT); a simulation of
// another method in a cluster plan is left untouched.
template <typename R, int M>
__global__ void __launch_bounds__(512) line_cluster_kernel(ion_line_plan plan, int mode, int n_steps) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cg::cluster_group cl = cg::this_cluster();
    const int C = int(cl.num_blocks());
    const int rank = int(cl.block_rank());
    ion_line_sim& S = plan.sims[blockIdx.x / C];
    const int64_t t0 = S.t, tf = S.t_final;
    const int n = S.n;
    const int T = (n + C * M - 1) / (C * M);
    if (n < 2 || n > plan.max_n || T > plan.threads || S.method == ION_LINE_FFT || S.gauge != ION_GAUGE_LENGTH)
        return;
    const int L = T * M, off = rank * L;
    Cx<R>* line = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* red = line + plan.threads * M;
    double* scratch = reinterpret_cast<double*>(red + 12 * plan.threads);
    double* part = scratch + 32;
    Cx<R>* g = static_cast<Cx<R>*>(S.g);
    const Cx<R> zero = {R(0), R(0)};

    if (mode == 1) {
        if (!line_is_data(t0, tf, S.store_every)) return;
        for (int i = threadIdx.x; i < L; i += blockDim.x) line[islot<M>(i, T)] = off + i < n ? ld(g + off + i) : zero;
        __syncthreads();
        line_reduce_cluster<R, M>(S, line, T, off, t0, scratch, part, rank, C);
        return;
    }
    const int64_t tend = tf - t0 > n_steps ? t0 + n_steps : tf;
    if (t0 >= tend) return;
    // Steps follow each other without a further cluster barrier: the
    // neighbours read this CTA's rows (halo, reduced system) only before the
    // barrier that ends each solve.
    for (int64_t t = t0; t < tend; ++t) {
    const LineTab<R> tb = LineTab<R>::make(S);
    const R tau = R(S.tau[t + 1]);
    const R ef = R(S.efield[t + 1]);
    const bool split = S.method == ION_LINE_SPLIT;

#pragma unroll
    for (int k = 0; k < M; ++k) {
        const int i = threadIdx.x + k * blockDim.x;
        if (i >= L) continue;
        const int gi = off + i;
        Cx<R> x = zero;
        if (gi < n) {
            x = ld(g + gi);
            if (split) x = phase(x, (tb.zq[gi] * ef) * tau);
        }
        line[islot<M>(i, T)] = x;
    }
    cl.sync();  // the neighbours' halo rows are staged
    const OffsetCoef<R> coef{LineCnCoef<R>{tb, tau, ef, !split, n}, off};
    const ClusterHalo<R> halo{rank > 0 ? cl.map_shared_rank(line, rank - 1) : nullptr,
                              rank + 1 < C ? cl.map_shared_rank(line, rank + 1) : nullptr};
    {
        const int tid = threadIdx.x;
        const bool active = tid < T;
        Cx<R> al[M], be[M], ga[M];
        RedRow<R> r[2];
        if (active) cn_chunk_eliminate<R, M>(T, tid, R(2), line, coef, NoExtra{}, al, be, ga, r[0], r[1], halo);
        pcr_solve_cluster<R>(T, tid, active, red, r, rank, C);
        if (active) {
            const LineAddOut<R, M> out{line, T};
            const int s = tid * M;
            const Cx<R> xs = r[0].d, xe = r[1].d;
            out(s, xs);
#pragma unroll
            for (int k = 1; k < M - 1; ++k) out(s + k, al[k] + be[k] * xs + ga[k] * xe);
            out(s + M - 1, xe);
        }
    }
    cl.sync();  // the solve's reads of the other CTAs' shared memory are done
    for (int i = threadIdx.x; i < L && off + i < n; i += blockDim.x) {
        const int gi = off + i;
        Cx<R>* p = line + islot<M>(i, T);
        Cx<R> x = *p;
        if (split) x = phase(x, (tb.zq[gi] * ef) * tau);
        if (tb.mask) x = Cx<R>{x.re * tb.mask[gi], x.im * tb.mask[gi]};
        *p = x;
        st(g + gi, x);
    }
    __syncthreads();
    if (line_is_data(t + 1, tf, S.store_every))
        line_reduce_cluster<R, M>(S, line, T, off, t + 1, scratch, part, rank, C);
    }
    // every CTA read S.t before the first cluster barrier above
    if (rank == 0 && threadIdx.x == 0) S.t = tend;
}

// ---------------------------------------------------------------------------
// Complex64 with a stored residual (ion_line_sim.g_lo, plan flag
// ION_LINE_RESIDUAL): psi = g + g_lo, FP32 arithmetic.  One kernel for every
// line length, launched as a cluster of C >= 1 CTAs with 8 rows per thread
// (three line buffers: psi, its residual, the increment).  Per step:
//   stage (g, g_lo) with the split operator's phase applied to the pair;
//   solve A Delta1 = -i 2 B psi with the explicit half in the exact-row-sum
//   difference form plus B g_lo, then refine: A delta = -i B (2 psi + Delta1)
//   - Delta1 (the same solver on phi = psi + Delta1 / 2, X = -i Delta1);
//   add Delta = Delta1 + delta to (g, g_lo) exactly, apply the phase and the
//   mask to the pair, store, and reduce g + g_lo in FP64 at data times.
// ---------------------------------------------------------------------------
constexpr int LINE_RES_M = 8;

__device__ __forceinline__ float two_sum_full(float a, float b, float& e) {
    const float s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
    return s;
}

// h + d with the residual lo: h + d formed exactly (Knuth's TwoSum), its
// rounding error added to lo, the pair renormalised (Fast2Sum); returns the
// new h and updates lo
__device__ __forceinline__ float add_exact1_f(float h, float d, float& lo) {
    float e;
    const float s = two_sum_full(h, d, e);
    const float l = lo + e;
    const float r = s + l;
    lo = l - (r - s);
    return r;
}
__device__ __forceinline__ Cx<float> add_exact_f(Cx<float> h, Cx<float> d, Cx<float>& lo) {
    return Cx<float>{add_exact1_f(h.re, d.re, lo.re), add_exact1_f(h.im, d.im, lo.im)};
}

// (hi + lo) * exp(-i theta), the rounding of hi's update kept in lo
__device__ __forceinline__ void phase_res(Cx<float>& hi, Cx<float>& lo, float theta) {
    float cm1, s;
    rot_coeffs(theta, cm1, s);
    float er, ei;
    const float hr = two_sum_full(hi.re, cm1 * hi.re + s * hi.im, er);
    const float hi_i = two_sum_full(hi.im, cm1 * hi.im - s * hi.re, ei);
    lo = Cx<float>{lo.re + (cm1 * lo.re + s * lo.im) + er, lo.im + (cm1 * lo.im - s * lo.re) + ei};
    hi = Cx<float>{hr, hi_i};
}

// (hi + lo) * m, the product's rounding kept in lo
__device__ __forceinline__ void scale_res(Cx<float>& hi, Cx<float>& lo, float m) {
    const float pr = hi.re * m, pi = hi.im * m;
    lo = Cx<float>{fmaf(lo.re, m, fmaf(hi.re, m, -pr)), fmaf(lo.im, m, fmaf(hi.im, m, -pi))};
    hi = Cx<float>{pr, pi};
}

// the line coefficients plus the staged residual (local rows; the rows just
// outside this CTA's segment come from the neighbouring CTAs' buffers)
template <int M>
struct LineResCoef {
    OffsetCoef<float> c;
    const Cx<float>* lob;
    const Cx<float>* prev;  // previous CTA's residual buffer (DSMEM) or nullptr
    const Cx<float>* next;
    const float* hd_lo;    // hd64 - hd32, the low part of the FP64 diagonal of H0, or NULL
    const float* hoff_lo;  // hoff64 - hoff32, or NULL
    float tau_lo;          // tau64 - tau32
    int T, L;
    __device__ __forceinline__ void operator()(int i, float& bo, float& bd) const { c(i, bo, bd); }
    // bd_exact - bd for the diagonal bd = tau * fma(zq, E, hd32) of local row
    // i: the rounding of hd32 from the FP64 diagonal (hd = -2p + V loses the
    // low bits of V beside the kinetic term, a random potential of ~1e-8 of
    // the kinetic diagonal) plus the rounding of the field term, of tau and
    // of the product with tau, formed with error-free transforms.  The
    // explicit half uses the exact diagonal; the refinement then solves with it.
    __device__ __forceinline__ float bd_lo(int i) const {
        const int gi = c.off + i;
        const LineCnCoef<float>& k = c.c;
        if (gi >= k.n) return 0.f;
        const float hd = k.tb.hd[gi];
        float h = hd, herr = hd_lo ? hd_lo[gi] : 0.f;
        if (k.with_field) {
            const float zq = k.tb.zq[gi];
            h = fmaf(zq, k.efield, hd);
            const float p = zq * k.efield;
            const float pe = fmaf(zq, k.efield, -p);
            float se;
            const float sm = two_sum_full(hd, p, se);
            herr += ((sm - h) + se) + pe;
        }
        const float b = k.tau * h;
        return fmaf(k.tau, h, -b) + fmaf(k.tau, herr, tau_lo * h);
    }
    // bo_exact - bo for the coupling of local rows i and i + 1 (0 outside
    // the line): the low parts of hoff and of tau, and the product's rounding
    __device__ __forceinline__ float bo_lo(int i) const {
        const int gi = c.off + i;
        const LineCnCoef<float>& k = c.c;
        if (gi < 0 || gi >= k.n - 1) return 0.f;
        const float o = k.tb.hoff[gi];
        return fmaf(k.tau, o, -(k.tau * o)) + fmaf(k.tau, hoff_lo ? hoff_lo[gi] : 0.f, tau_lo * o);
    }
    __device__ __forceinline__ Cx<float> lo_at(int i) const {
        if (i < 0) return prev ? prev[islot<M>(L - 1, T)] : Cx<float>{0.f, 0.f};
        if (i >= L) return next ? next[0] : Cx<float>{0.f, 0.f};
        return lob[islot<M>(i, T)];
    }
};

template <int M>
__device__ __forceinline__ Cx<float> stencil_row(const LineResCoef<M>& c, int i, float a0, float bd, float bo,
                                                  Cx<float> p0, Cx<float> p1, Cx<float> p2) {
    float e1, e2;
    const float s1 = two_sum_full(bd, a0, e1);
    const float rs = two_sum_full(s1, bo, e2);
    // the remainders of the FP64 diagonal and couplings enter the row sum;
    // the couplings' own roundings act on neighbour differences only, which
    // matters far less (a relative error of ~1e-7 in the kinetic energy)
    const float rl = ((e1 + e2) + c.bd_lo(i)) + (c.bo_lo(i - 1) + c.bo_lo(i));
    const Cx<float> dm = p0 - p1, dp = p2 - p1;
    const Cx<float> l0 = c.lo_at(i - 1), l1 = c.lo_at(i), l2 = c.lo_at(i + 1);
    return Cx<float>{a0 * dm.re + bo * dp.re + (rs * p1.re + rl * p1.re) + (a0 * l0.re + bd * l1.re + bo * l2.re),
                     a0 * dm.im + bo * dp.im + (rs * p1.im + rl * p1.im) + (a0 * l0.im + bd * l1.im + bo * l2.im)};
}

// X_i = -i d_i from an interleaved buffer, or 0
template <int M>
struct LineMinusIExtra {
    const Cx<float>* d;
    int T;
    bool on;
    template <typename RR>
    __device__ __forceinline__ Cx<RR> get(int i) const {
        if (!on) return Cx<RR>{RR(0), RR(0)};
        const Cx<float> v = d[islot<M>(i, T)];
        return Cx<RR>{v.im, -v.re};
    }
};

template <int M>
struct LineSetAddOut {
    Cx<float>* line;
    int T;
    bool add;
    __device__ __forceinline__ void operator()(int i, Cx<float> d) const {
        Cx<float>* p = line + islot<M>(i, T);
        *p = add ? *p + d : d;
    }
};

// norm and inner products of hi + lo over the cluster
template <int M>
__device__ void line_reduce_res(const ion_line_sim& S, const Cx<float>* line, const Cx<float>* lob, int T, int off,
                                int64_t t, double* scratch, double* part, int rank, int C) {
    const int n = S.n;
    const int L = T * M;
    const int64_t slot = line_slot(t, S.t_final, S.store_every);
    const int i0 = int(threadIdx.x) < T ? int(threadIdx.x) : L;
    auto val = [&](int i) {
        const Cx<float> h = line[islot<M>(i, T)], l = lob[islot<M>(i, T)];
        return Cx<double>{double(h.re) + double(l.re), double(h.im) + double(l.im)};
    };
    double acc = 0.0;
    for (int i = i0; i < L && off + i < n; i += T) {
        const Cx<double> x = val(i);
        acc += x.re * x.re + x.im * x.im;
    }
    double nrm = block_sum_l(acc, scratch), unused = 0.0;
    cluster_sum2(nrm, unused, part, 0, rank, C);
    if (rank == 0 && threadIdx.x == 0) S.out_norm[slot] = nrm * S.weight;
    for (int s = 0; s < S.n_states; ++s) {
        const double* sg = S.state_g + int64_t(s) * n * 2;
        double re = 0.0, im = 0.0;
        for (int i = i0; i < L && off + i < n; i += T) {
            const Cx<double> x = val(i);
            const double ar = sg[2 * (off + i)], ai = -sg[2 * (off + i) + 1];
            re += ar * x.re - ai * x.im;
            im += ar * x.im + ai * x.re;
        }
        double tr = block_sum_l(re, scratch);
        double ti = block_sum_l(im, scratch);
        cluster_sum2(tr, ti, part, s + 1, rank, C);
        if (rank == 0 && threadIdx.x == 0) {
            S.out_ip[(slot * S.n_states + s) * 2] = tr * S.weight;
            S.out_ip[(slot * S.n_states + s) * 2 + 1] = ti * S.weight;
        }
    }
}

__host__ __device__ inline size_t line_res_smem(int threads) {
    return 3 * size_t(threads) * LINE_RES_M * sizeof(Cx<float>) + pcr_smem_bytes<float>(threads) +
           64 * sizeof(double);
}

// Crank-Nicolson methods (ION_LINE_ADI / ION_LINE_SPLIT) with a residual; a
// simulation of another method, or without g_lo, is left untouched.
__global__ void __launch_bounds__(512) line_res_kernel(ion_line_plan plan, int mode, int n_steps) {
    constexpr int M = LINE_RES_M;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cg::cluster_group cl = cg::this_cluster();
    const int C = int(cl.num_blocks());
    const int rank = int(cl.block_rank());
    ion_line_sim& S = plan.sims[blockIdx.x / C];
    const int64_t t0 = S.t, tf = S.t_final;
    const int n = S.n;
    const int T = (n + C * M - 1) / (C * M);
    if (n < 2 || n > plan.max_n || T > plan.threads || S.method == ION_LINE_FFT || S.g_lo == nullptr ||
        S.gauge != ION_GAUGE_LENGTH)
        return;
    const int L = T * M, off = rank * L;
    const int cap = plan.threads * M;
    Cx<float>* line = reinterpret_cast<Cx<float>*>(smem_raw);
    Cx<float>* lob = line + cap;
    Cx<float>* ext = lob + cap;
    Cx<float>* red = ext + cap;
    double* scratch = reinterpret_cast<double*>(red + 12 * plan.threads);
    double* part = scratch + 32;
    Cx<float>* g = static_cast<Cx<float>*>(S.g);
    uint32_t* glo = static_cast<uint32_t*>(S.g_lo);  // packed bf16x2
    const Cx<float> zero = {0.f, 0.f};

    if (mode == 1) {
        if (!line_is_data(t0, tf, S.store_every)) return;
        for (int i = threadIdx.x; i < L; i += blockDim.x) {
            const bool in = off + i < n;
            line[islot<M>(i, T)] = in ? ld(g + off + i) : zero;
            lob[islot<M>(i, T)] = in ? lo_unpack(glo[off + i]) : zero;
        }
        __syncthreads();
        line_reduce_res<M>(S, line, lob, T, off, t0, scratch, part, rank, C);
        return;
    }
    const int64_t tend = tf - t0 > n_steps ? t0 + n_steps : tf;
    if (t0 >= tend) return;
    // as in line_cluster_kernel, the neighbours are done with this CTA's rows
    // at the barrier that ends the second solve of a step
    for (int64_t t = t0; t < tend; ++t) {
    const LineTab<float> tb = LineTab<float>::make(S);
    const float tau = float(S.tau[t + 1]);
    const float ef = float(S.efield[t + 1]);
    const bool split = S.method == ION_LINE_SPLIT;
    // the pair at global row gi as staged: (g, g_lo) with the first phase
    auto staged = [&](int gi, Cx<float>& h, Cx<float>& lw) {
        h = ld(g + gi);
        lw = lo_unpack(glo[gi]);
        if (split) phase_res(h, lw, (tb.zq[gi] * ef) * tau);
    };
    for (int i = threadIdx.x; i < L; i += blockDim.x) {
        Cx<float> h = zero, lw = zero;
        if (off + i < n) staged(off + i, h, lw);
        line[islot<M>(i, T)] = h;
        lob[islot<M>(i, T)] = lw;
    }
    cl.sync();  // the neighbours' halo rows are staged
    const LineResCoef<M> coef{OffsetCoef<float>{LineCnCoef<float>{tb, tau, ef, !split, n}, off}, lob,
                              rank > 0 ? cl.map_shared_rank(lob, rank - 1) : nullptr,
                              rank + 1 < C ? cl.map_shared_rank(lob, rank + 1) : nullptr, S.hd_lo32, S.hoff_lo32,
                              float(S.tau[t + 1] - double(tau)), T, L};
    const ClusterHalo<float> halo{rank > 0 ? cl.map_shared_rank(line, rank - 1) : nullptr,
                                  rank + 1 < C ? cl.map_shared_rank(line, rank + 1) : nullptr};
    const int tid = threadIdx.x;
    const bool active = tid < T;
    for (int pass = 0; pass < 2; ++pass) {
        {
            Cx<float> al[M], be[M], ga[M];
            RedRow<float> r[2];
            if (active)
                cn_chunk_eliminate<float, M>(T, tid, 2.f, line, coef, LineMinusIExtra<M>{ext, T, pass == 1}, al, be,
                                             ga, r[0], r[1], halo);
            if (C == 1)  // one CTA: the halved block PCR with CTA barriers
                pcr_solve_cn<float>(T, tid, active, red, r);
            else
                pcr_solve_cluster<float>(T, tid, active, red, r, rank, C);
            if (active) {
                const LineSetAddOut<M> out{ext, T, pass == 1};
                const int s = tid * M;
                const Cx<float> xs = r[0].d, xe = r[1].d;
                out(s, xs);
#pragma unroll
                for (int k = 1; k < M - 1; ++k) out(s + k, al[k] + be[k] * xs + ga[k] * xe);
                out(s + M - 1, xe);
            }
        }
        if (C > 1)
            cl.sync();  // the solve's reads of the other CTAs' shared memory are done
        else
            __syncthreads();
        if (pass == 0) {  // phi = psi + Delta1 / 2
            for (int i = threadIdx.x; i < L; i += blockDim.x) {
                const int sl = islot<M>(i, T);
                line[sl] = line[sl] + scale(ext[sl], 0.5f);
            }
            cl.sync();  // the neighbours read this CTA's phi as their halo
        }
    }
    for (int i = threadIdx.x; i < L && off + i < n; i += blockDim.x) {
        const int gi = off + i;
        const int sl = islot<M>(i, T);
        Cx<float> h, lw;
        staged(gi, h, lw);
        h = add_exact_f(h, ext[sl], lw);
        if (split) phase_res(h, lw, (tb.zq[gi] * ef) * tau);
        if (tb.mask) scale_res(h, lw, tb.mask[gi]);
        // the residual as stored (packed): the data reductions below see what
        // the next step reloads
        const uint32_t w = lo_pack(lw);
        line[sl] = h;
        lob[sl] = lo_unpack(w);
        st(g + gi, h);
        glo[gi] = w;
    }
    __syncthreads();
    if (line_is_data(t + 1, tf, S.store_every)) line_reduce_res<M>(S, line, lob, T, off, t + 1, scratch, part, rank, C);
    }
    // every CTA read S.t before the first cluster barrier above
    if (rank == 0 && threadIdx.x == 0) S.t = tend;
}

constexpr int LINE_MAX_CLUSTER = 8;
constexpr size_t LINE_SMEM_LIMIT = 200 * 1024;

template <typename R>
static bool line_residual(const ion_line_plan* p) {
    return std::is_same<R, float>::value && p && (p->flags & ION_LINE_RESIDUAL);
}

static int line_res_validate(const ion_line_plan* p) {
    if (!p->sims || p->n_sims < 0 || p->max_n < 2 || p->threads <= 0 || p->threads > 512 || (p->threads & 31) ||
        p->cluster < 0 || p->cluster > LINE_MAX_CLUSTER) {
        set_error("ion_line: invalid plan");
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int C = p->cluster > 1 ? p->cluster : 1;
    if (line_threads(p->max_n, C * LINE_RES_M) > p->threads) {
        set_error("ion_line: max_n = %d needs more than %d threads x %d CTAs", p->max_n, p->threads, C);
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (line_res_smem(p->threads) > LINE_SMEM_LIMIT) {
        set_error("ion_line: line too long for shared memory");
        return ION_ERR_UNSUPPORTED;
    }
    return ION_OK;
}

static int line_res_launch(const ion_line_plan* p, int mode, int n_steps, cudaStream_t s) {
    if (int e = ensure_smem_limit((const void*)line_res_kernel, int(LINE_SMEM_LIMIT), "line_res_kernel")) return e;
    const unsigned C = unsigned(p->cluster > 1 ? p->cluster : 1);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(unsigned(p->n_sims) * C);
    cfg.blockDim = dim3(unsigned(p->threads));
    cfg.dynamicSmemBytes = line_res_smem(p->threads);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int active = 0;
    if (cudaOccupancyMaxActiveClusters(&active, line_res_kernel, &cfg) != cudaSuccess || active < 1) {
        cudaGetLastError();
        set_error("ion_line: a cluster of %u CTAs x %d threads does not fit on the device", C, p->threads);
        return ION_ERR_UNSUPPORTED;
    }
    cudaLaunchKernelEx(&cfg, line_res_kernel, *p, mode, n_steps);
    return check_launch("line_res_kernel");
}

template <typename R>
static int line_validate(const ion_line_plan* p) {
    constexpr int M = LineCfg<R>::M;
    if (line_residual<R>(p)) return line_res_validate(p);
    if (!p || !p->sims || p->n_sims < 0 || p->max_n < 2 || p->threads <= 0 || p->threads > LineCfg<R>::MAX_T ||
        (p->threads & 31) || p->cluster < 0 || p->cluster > LINE_MAX_CLUSTER) {
        set_error("ion_line: invalid plan");
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int C = p->cluster > 1 ? p->cluster : 1;
    if (line_threads(p->max_n, C * M) > p->threads) {
        set_error("ion_line: max_n = %d needs more than %d threads x %d CTAs", p->max_n, p->threads, C);
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (line_cluster_smem<R>(p->threads, M) > LINE_SMEM_LIMIT ||
        line_smem<R>(p->threads, M, (p->flags & ION_LINE_HAS_FFT) != 0) > LINE_SMEM_LIMIT) {
        set_error("ion_line: line too long for shared memory");
        return ION_ERR_UNSUPPORTED;
    }
    return ION_OK;
}

template <typename R>
static int line_launch(const ion_line_plan* p, int mode, int n_steps, cudaStream_t s) {
    constexpr int M = LineCfg<R>::M;
    if (line_residual<R>(p)) return line_res_launch(p, mode, n_steps, s);
    if (p->cluster > 1) {
        auto k = line_cluster_kernel<R, M>;
        if (int e = ensure_smem_limit((const void*)k, int(LINE_SMEM_LIMIT), "line_cluster_kernel")) return e;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(unsigned(p->n_sims) * unsigned(p->cluster));
        cfg.blockDim = dim3(unsigned(p->threads));
        cfg.dynamicSmemBytes = line_cluster_smem<R>(p->threads, M);
        cfg.stream = s;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = unsigned(p->cluster);
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int active = 0;
        if (cudaOccupancyMaxActiveClusters(&active, k, &cfg) != cudaSuccess || active < 1) {
            cudaGetLastError();
            set_error("ion_line: a cluster of %d CTAs x %d threads does not fit on the device", p->cluster,
                      p->threads);
            return ION_ERR_UNSUPPORTED;
        }
        cudaLaunchKernelEx(&cfg, k, *p, mode, n_steps);
        return check_launch("line_cluster_kernel");
    }
    if (int e = ensure_smem_limit((const void*)line_step_kernel<R, M>, int(LINE_SMEM_LIMIT), "line_step_kernel"))
        return e;
    line_step_kernel<R, M><<<p->n_sims, p->threads,
                             line_smem<R>(p->threads, M, (p->flags & ION_LINE_HAS_FFT) != 0), s>>>(*p, mode, n_steps);
    return check_launch("line_step_kernel");
}

template <typename R>
static int line_run(const ion_line_plan* p, int64_t n_steps, void* stream) {
    if (int e = line_validate<R>(p)) return e;
    if (n_steps < 0) {
        set_error("ion_line: negative step count");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (p->n_sims == 0) return ION_OK;
    cudaStream_t s = as_stream(stream);
    // one launch advances every line by up to 2^30 steps (each CTA loops over
    // the steps; a line that reaches t_final stops there)
    for (int64_t done = 0; done < n_steps;) {
        const int k = int(n_steps - done < (int64_t(1) << 30) ? n_steps - done : (int64_t(1) << 30));
        if (int e = line_launch<R>(p, 0, k, s)) return e;
        done += k;
    }
    return ION_OK;
}

template <typename R>
static int line_reduce_only(const ion_line_plan* p, void* stream) {
    if (int e = line_validate<R>(p)) return e;
    if (p->n_sims == 0) return ION_OK;
    return line_launch<R>(p, 1, 0, as_stream(stream));
}

template <typename R>
static int64_t line_max_n() {
    constexpr int M = LineCfg<R>::M;
    int T = LineCfg<R>::MAX_T;
    while (T > 32 && line_cluster_smem<R>(T, M) > LINE_SMEM_LIMIT) T -= 32;
    return int64_t(T) * M;
}

}  // namespace ion

using namespace ion;

extern "C" {
int ion_line_run_c128(const ion_line_plan* plan, int64_t n_steps, void* stream) {
    return line_run<double>(plan, n_steps, stream);
}
int ion_line_run_c64(const ion_line_plan* plan, int64_t n_steps, void* stream) {
    return line_run<float>(plan, n_steps, stream);
}
int ion_line_reduce_c128(const ion_line_plan* plan, void* stream) { return line_reduce_only<double>(plan, stream); }
int ion_line_reduce_c64(const ion_line_plan* plan, void* stream) { return line_reduce_only<float>(plan, stream); }
int64_t ion_line_max_n_c128(void) { return line_max_n<double>(); }
int64_t ion_line_max_n_c64(void) { return line_max_n<float>(); }
int64_t ion_line_max_n_c64x(void) {
    int T = 512;
    while (T > 32 && line_res_smem(T) > LINE_SMEM_LIMIT) T -= 32;
    return int64_t(T) * LINE_RES_M;
}
}
