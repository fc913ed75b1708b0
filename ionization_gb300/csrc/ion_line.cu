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
#include "ion_common.cuh"
#include "ion_cn_solver.cuh"

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
        const R h = with_field ? tb.hd[i] + tb.zq[i] * efield : tb.hd[i];
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

// norm and inner products of the line held in shared memory (FP64)
template <typename R, int M>
__device__ void line_reduce(const ion_line_sim& S, const Cx<R>* line, int T, int64_t t, double* scratch) {
    const int n = S.n;
    const int64_t slot = line_slot(t, S.t_final, S.store_every);
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const Cx<R> x = line[islot<M>(i, T)];
        acc += double(x.re) * double(x.re) + double(x.im) * double(x.im);
    }
    const double nrm = block_sum_l(acc, scratch);
    if (threadIdx.x == 0) S.out_norm[slot] = nrm * S.weight;
    for (int s = 0; s < S.n_states; ++s) {
        const double* sg = S.state_g + int64_t(s) * n * 2;
        double re = 0.0, im = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
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

template <typename R>
__host__ __device__ inline size_t line_smem(int threads, int M) {
    return size_t(threads) * M * sizeof(Cx<R>) + pcr_smem_bytes<R>(threads) + 32 * sizeof(double);
}

// mode 0: one step (t -> t+1) then reduce if data time; mode 1: reduce at t only
template <typename R, int M>
__global__ void __launch_bounds__(512) line_step_kernel(ion_line_plan plan, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ion_line_sim& S = plan.sims[blockIdx.x];
    const int64_t t = S.t, tf = S.t_final;
    const int n = S.n;
    const int T = line_threads(n, M);
    const int npad = T * M;
    Cx<R>* line = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* red = line + plan.threads * M;
    double* scratch = reinterpret_cast<double*>(red + 12 * plan.threads);
    Cx<R>* g = static_cast<Cx<R>*>(S.g);
    const Cx<R> zero = {R(0), R(0)};

    if (mode == 1) {
        if (!line_is_data(t, tf, S.store_every)) return;
        for (int i = threadIdx.x; i < n; i += blockDim.x) line[islot<M>(i, T)] = ld(g + i);
        __syncthreads();
        line_reduce<R, M>(S, line, T, t, scratch);
        return;
    }
    if (t >= tf) return;
    const LineTab<R> tb = LineTab<R>::make(S);
    const R tau = R(S.tau[t + 1]);
    const R ef = R(S.efield[t + 1]);
    const bool split = S.method == ION_LINE_SPLIT;

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
    const LineCnCoef<R> coef{tb, tau, ef, !split, n};
    block_cn_solve<R, M>(T, threadIdx.x, R(2), line, red, coef, NoExtra{}, LineAddOut<R, M>{line, T});
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Cx<R>* p = line + islot<M>(i, T);
        Cx<R> x = *p;
        if (split) x = phase(x, (tb.zq[i] * ef) * tau);
        if (tb.mask) x = Cx<R>{x.re * tb.mask[i], x.im * tb.mask[i]};
        *p = x;
        st(g + i, x);
    }
    __syncthreads();
    if (line_is_data(t + 1, tf, S.store_every)) line_reduce<R, M>(S, line, T, t + 1, scratch);
    __syncthreads();
    if (threadIdx.x == 0) S.t = t + 1;
}

template <typename R>
static int line_validate(const ion_line_plan* p) {
    constexpr int M = LineCfg<R>::M;
    if (!p || !p->sims || p->n_sims < 0 || p->max_n < 2 || p->threads <= 0 || p->threads > LineCfg<R>::MAX_T ||
        (p->threads & 31) || line_threads(p->max_n, M) > p->threads) {
        set_error("ion_line: invalid plan");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (line_smem<R>(p->threads, M) > 200 * 1024) {
        set_error("ion_line: line too long for shared memory");
        return ION_ERR_UNSUPPORTED;
    }
    return ION_OK;
}

template <typename R>
static int line_launch(const ion_line_plan* p, int mode, cudaStream_t s) {
    constexpr int M = LineCfg<R>::M;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(line_step_kernel<R, M>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    line_step_kernel<R, M><<<p->n_sims, p->threads, line_smem<R>(p->threads, M), s>>>(*p, mode);
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
    for (int64_t k = 0; k < n_steps; ++k)
        if (int e = line_launch<R>(p, 0, s)) return e;
    return ION_OK;
}

template <typename R>
static int line_reduce_only(const ion_line_plan* p, void* stream) {
    if (int e = line_validate<R>(p)) return e;
    if (p->n_sims == 0) return ION_OK;
    return line_launch<R>(p, 1, as_stream(stream));
}

template <typename R>
static int64_t line_max_n() {
    constexpr int M = LineCfg<R>::M;
    int T = LineCfg<R>::MAX_T;
    while (T > 32 && line_smem<R>(T, M) > 200 * 1024) T -= 32;
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
}
