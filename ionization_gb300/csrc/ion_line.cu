// Line mesh, length gauge: LineMesh (ionization/mesh/meshes.py:263-341) with
// LineLengthGaugeOperators (ionization/mesh/mesh_operators.py:304-341) under
// AlternatingDirectionImplicit or SplitInteractionOperator
// (ionization/mesh/evolution_methods.py:46-123), then the mask
// (meshes.py:256-257).
//
// One CTA owns one simulation for a whole step: psi is staged in shared
// memory, the explicit half-step is formed on the fly, the implicit half-step
// is the block partition + PCR solve, then the mask and (at data times) the
// norm / inner products are reduced from shared memory before psi is stored.
#include "ion_common.cuh"
#include "ion_solver.cuh"

namespace ion {

template <typename R> struct LineCfg;
template <> struct LineCfg<double> {
    static constexpr int MAXM = 8;
    static constexpr int MAX_T = 512;
};
template <> struct LineCfg<float> {
    static constexpr int MAXM = 16;
    static constexpr int MAX_T = 512;
};

__host__ __device__ inline int line_threads(int n, int maxm) {
    int T = (n + maxm - 1) / maxm;
    if (T > n / 2) T = n / 2;
    if (T < 1) T = 1;
    return T;
}

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

// H diagonal at row i: H0 + (zq * E) for ADI, H0 for split
template <typename R>
struct LineH {
    LineTab<R> tb;
    R efield;
    bool with_field;
    __device__ R diag(int i) const { return with_field ? tb.hd[i] + tb.zq[i] * efield : tb.hd[i]; }
    __device__ R off(int i) const { return tb.hoff[i]; }
};

template <typename R>
struct LineCoef {
    LineH<R> h;
    R tau;
    int n;
    __device__ void operator()(int64_t i, Cx<R>& a, Cx<R>& b, Cx<R>& c) const {
        const Cx<R> zero = {R(0), R(0)};
        a = (i > 0) ? Cx<R>{R(0), tau * h.off(int(i) - 1)} : zero;
        b = Cx<R>{R(1), tau * h.diag(int(i))};
        c = (i < n - 1) ? Cx<R>{R(0), tau * h.off(int(i))} : zero;
    }
};

template <typename R>
struct LineExplicit {
    LineH<R> h;
    R tau;
    int n;
    const Cx<R>* psi;
    __device__ Cx<R> operator()(int64_t i_) const {
        const int i = int(i_);
        Cx<R> y = {R(0), R(0)};
        if (i > 0) y = mul_ih(-tau * h.off(i - 1), psi[i - 1]);
        const Cx<R> p = psi[i];
        const R hd = -tau * h.diag(i);
        y = y + Cx<R>{p.re - hd * p.im, p.im + hd * p.re};
        if (i < n - 1) y = y + mul_ih(-tau * h.off(i), psi[i + 1]);
        return y;
    }
};

template <typename R>
struct LineOut {
    Cx<R>* line;
    __device__ void operator()(int64_t i, Cx<R> x) const { line[i] = x; }
};

__device__ __forceinline__ void sincos_l(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sincos_l(float x, float* s, float* c) { sincosf(x, s, c); }

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

// norm and inner products of the line in shared memory (FP64)
template <typename R>
__device__ void line_reduce(const ion_line_sim& S, const Cx<R>* line, int64_t t, double* scratch) {
    const int n = S.n;
    const int64_t slot = line_slot(t, S.t_final, S.store_every);
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const Cx<R> x = line[i];
        acc += double(x.re) * double(x.re) + double(x.im) * double(x.im);
    }
    const double nrm = block_sum_l(acc, scratch);
    if (threadIdx.x == 0) S.out_norm[slot] = nrm * S.weight;
    for (int s = 0; s < S.n_states; ++s) {
        const double* sg = S.state_g + int64_t(s) * n * 2;
        double re = 0.0, im = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const Cx<R> x = line[i];
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
__host__ __device__ inline size_t line_smem(int max_n, int threads) {
    return (size_t(max_n) + 1) / 2 * 2 * sizeof(Cx<R>) + pcr_smem_bytes<R>(threads) + 32 * sizeof(double);
}

// mode 0: one step (t -> t+1) then reduce if data time; mode 1: reduce at t only
template <typename R, int MAXM>
__global__ void __launch_bounds__(512) line_step_kernel(ion_line_plan plan, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ion_line_sim& S = plan.sims[blockIdx.x];
    const int64_t t = S.t, tf = S.t_final;
    const int n = S.n;
    Cx<R>* line = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* red = line + (plan.max_n + 1) / 2 * 2;
    double* scratch = reinterpret_cast<double*>(red + 12 * plan.threads);
    Cx<R>* g = static_cast<Cx<R>*>(S.g);

    if (mode == 1) {
        if (!line_is_data(t, tf, S.store_every)) return;
        for (int i = threadIdx.x; i < n; i += blockDim.x) line[i] = ld(g + i);
        __syncthreads();
        line_reduce<R>(S, line, t, scratch);
        return;
    }
    if (t >= tf) return;
    const LineTab<R> tb = LineTab<R>::make(S);
    const R tau = R(S.tau[t + 1]);
    const R ef = R(S.efield[t + 1]);
    const bool split = S.method == ION_LINE_SPLIT;

    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Cx<R> x = ld(g + i);
        if (split) {  // exp(-i tau zq E)
            R s, c;
            sincos_l(tb.zq[i] * ef * tau, &s, &c);
            x = Cx<R>{c * x.re + s * x.im, c * x.im - s * x.re};
        }
        line[i] = x;
    }
    __syncthreads();
    const int T = line_threads(n, MAXM);
    const LineH<R> h{tb, ef, !split};
    block_line_solve<R, MAXM>(n, T, threadIdx.x, int(threadIdx.x) < T, red, LineCoef<R>{h, tau, n},
                              LineExplicit<R>{h, tau, n, line}, LineOut<R>{line});
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Cx<R> x = line[i];
        if (split) {
            R s, c;
            sincos_l(tb.zq[i] * ef * tau, &s, &c);
            x = Cx<R>{c * x.re + s * x.im, c * x.im - s * x.re};
        }
        if (tb.mask) x = Cx<R>{x.re * tb.mask[i], x.im * tb.mask[i]};
        line[i] = x;
        st(g + i, x);
    }
    __syncthreads();
    if (line_is_data(t + 1, tf, S.store_every)) line_reduce<R>(S, line, t + 1, scratch);
    __syncthreads();
    if (threadIdx.x == 0) S.t = t + 1;
}

template <typename R>
static int line_validate(const ion_line_plan* p) {
    constexpr int MAXM = LineCfg<R>::MAXM;
    if (!p || !p->sims || p->n_sims < 0 || p->max_n < 2 || p->threads <= 0 ||
        p->threads > LineCfg<R>::MAX_T || (p->threads & 31) ||
        int64_t(p->max_n) > int64_t(MAXM) * LineCfg<R>::MAX_T ||
        line_threads(p->max_n, MAXM) > p->threads) {
        set_error("ion_line: invalid plan");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (line_smem<R>(p->max_n, p->threads) > 200 * 1024) {
        set_error("ion_line: line too long for shared memory");
        return ION_ERR_UNSUPPORTED;
    }
    return ION_OK;
}

template <typename R>
static int line_launch(const ion_line_plan* p, int mode, cudaStream_t s) {
    constexpr int MAXM = LineCfg<R>::MAXM;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(line_step_kernel<R, MAXM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             200 * 1024);
        attr = true;
    }
    line_step_kernel<R, MAXM><<<p->n_sims, p->threads, line_smem<R>(p->max_n, p->threads), s>>>(*p, mode);
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
int64_t ion_line_max_n_c128(void) {
    int64_t n = int64_t(LineCfg<double>::MAXM) * LineCfg<double>::MAX_T;
    while (line_smem<double>(int(n), LineCfg<double>::MAX_T) > 200 * 1024) n -= 64;
    return n;
}
int64_t ion_line_max_n_c64(void) {
    int64_t n = int64_t(LineCfg<float>::MAXM) * LineCfg<float>::MAX_T;
    while (line_smem<float>(int(n), LineCfg<float>::MAX_T) > 200 * 1024) n -= 64;
    return n;
}
}
