// Spherical-harmonic (l, r) mesh, length gauge, split-interaction operator.
//
// Reference path: SplitInteractionOperator.get_evolution_operators
// (ionization/mesh/evolution_methods.py:89-123) over
// SphericalHarmonicLengthGaugeOperators (ionization/mesh/mesh_operators.py:
// 815-1080), applied by QuantumMesh.evolve (ionization/mesh/meshes.py:251-257)
// once per step of MeshSimulation.run (ionization/mesh/sims.py:289-333).
//
// Per step three kernels run on the whole batch:
//   sh_cn_kernel   one CTA per (simulation, l) radial line: the line is staged
//                  in shared memory, y = (1 - i tau H0) psi is formed on the
//                  fly and (1 + i tau H0) x = y is solved by the block
//                  partition + PCR solver;
//   sh_rot_kernel  one CTA per (simulation, tile of r rows) holding all l of
//                  those rows: the rotations after the radial solve of step
//                  t+1 (odd, even), the mask, the data-time reductions, and
//                  the rotations before the radial solve of step t+2 (even,
//                  odd), all fused in one pass;
//   sh_advance_kernel  finishes the reductions (compensated sum over tiles)
//                  and advances each simulation's time index.
#include <cstdio>

#include "ion_common.cuh"
#include "ion_solver.cuh"

namespace ion {

enum : int { ROT_PRE_ONLY = 1, ROT_STEP = 2, ROT_STEP_PRE = 3, ROT_REDUCE_ONLY = 4 };
enum : int { ADV_STEP = 1, ADV_FINALIZE = 2 };

template <typename R> struct ShCfg;
template <> struct ShCfg<double> {
    static constexpr int MAXM = 8;
    static constexpr int MAX_T = 512;
};
template <> struct ShCfg<float> {
    static constexpr int MAXM = 16;
    static constexpr int MAX_T = 512;
};

__host__ __device__ inline int sh_line_threads(int nr, int maxm) {
    int T = (nr + maxm - 1) / maxm;
    if (T > nr / 2) T = nr / 2;
    if (T < 1) T = 1;
    return T;
}

__host__ __device__ inline bool is_data_time(int64_t t, int64_t t_final, int64_t every) {
    return t == 0 || t == t_final || (every >= 1 && t % every == 0);
}

__host__ __device__ inline int64_t data_slot(int64_t t, int64_t t_final, int64_t every) {
    if (every >= 1) return (t % every == 0) ? t / every : t_final / every + 1;
    return t == 0 ? 0 : 1;
}

// ---------------------------------------------------------------------------
// coefficients: A = 1 + i tau H on row i of line l
// ---------------------------------------------------------------------------
template <typename R> struct ShH;

template <> struct ShH<double> {  // exact FP64 tables
    const double* hd;               // row l of the diagonal table
    const double* hoff;
    __device__ double diag(int i) const { return hd[i]; }
    __device__ double off(int i) const { return hoff[i]; }  // couples i and i+1
    __device__ static ShH make(const ion_sh_sim& S, int l) { return ShH{S.hd + int64_t(l) * S.n_r, S.hoff}; }
};

template <> struct ShH<float> {  // FP32 tables rounded from FP64
    const float* kinv;
    const float* cent;
    const float* hoff;
    float ll1;
    float corr0;
    __device__ float diag(int i) const {
        float h = kinv[i] + ll1 * cent[i];
        return (i == 0) ? h + corr0 : h;
    }
    __device__ float off(int i) const { return hoff[i]; }
    __device__ static ShH make(const ion_sh_sim& S, int l) {
        return ShH{S.kinv32, S.cent32, S.hoff32, float(l) * float(l + 1), (l == 0) ? S.corr0_32 : 0.f};
    }
};

template <typename R>
struct ShCoef {
    ShH<R> h;
    R tau;
    int n;
    __device__ void operator()(int64_t i, Cx<R>& a, Cx<R>& b, Cx<R>& c) const {
        const Cx<R> zero = {R(0), R(0)};
        a = (i > 0) ? Cx<R>{R(0), tau * h.off(int(i) - 1)} : zero;
        b = Cx<R>{R(1), tau * h.diag(int(i))};
        c = (i < n - 1) ? Cx<R>{R(0), tau * h.off(int(i))} : zero;
    }
};

// y_i = ((1 - i tau H) psi)_i with psi staged in shared memory; terms are
// accumulated sub, diag, super as in the dia-matrix product
template <typename R>
struct ShExplicit {
    ShH<R> h;
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
struct SmemOut {
    Cx<R>* line;
    __device__ void operator()(int64_t i, Cx<R> x) const { line[i] = x; }
};

template <typename R>
__host__ __device__ inline size_t sh_cn_smem(int max_nr, int threads) {
    return (size_t(max_nr) + 1) / 2 * 2 * sizeof(Cx<R>) + pcr_smem_bytes<R>(threads);
}

template <typename R, int MAXM>
__global__ void __launch_bounds__(512) sh_cn_kernel(ion_sh_plan plan) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int item = blockIdx.x;
    const int si = plan.cn_items[2 * item];
    const int l = plan.cn_items[2 * item + 1];
    const ion_sh_sim& S = plan.sims[si];
    const int64_t t = S.t;
    if (t >= S.t_final) return;  // whole CTA leaves together
    const int nr = S.n_r;
    const int T = sh_line_threads(nr, MAXM);
    Cx<R>* line = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* red = line + (plan.max_n_r + 1) / 2 * 2;
    Cx<R>* g = static_cast<Cx<R>*>(S.g) + int64_t(l) * nr;
    for (int i = threadIdx.x; i < nr; i += blockDim.x) line[i] = ld(g + i);
    __syncthreads();
    const R tau = R(S.tau[t + 1]);
    const ShH<R> h = ShH<R>::make(S, l);
    ShCoef<R> coef{h, tau, nr};
    ShExplicit<R> rhs{h, tau, nr, line};
    block_line_solve<R, MAXM>(nr, T, threadIdx.x, int(threadIdx.x) < T, red, coef, rhs, SmemOut<R>{line});
    __syncthreads();
    for (int i = threadIdx.x; i < nr; i += blockDim.x) st(g + i, line[i]);
}

// ---------------------------------------------------------------------------
// rotation / mask / reduction pass over tiles of r rows
// ---------------------------------------------------------------------------
template <typename R>
struct RotTab;
template <> struct RotTab<double> {
    const double* cl;
    const double* rq;
    const double* mask;
    __device__ static RotTab make(const ion_sh_sim& S) { return RotTab{S.cl, S.rq, S.mask}; }
};
template <> struct RotTab<float> {
    const float* cl;
    const float* rq;
    const float* mask;
    __device__ static RotTab make(const ion_sh_sim& S) { return RotTab{S.cl32, S.rq32, S.mask32}; }
};

__device__ __forceinline__ void sincos_r(double x, double* s, double* c) { sincos(x, s, c); }
__device__ __forceinline__ void sincos_r(float x, float* s, float* c) { sincosf(x, s, c); }

constexpr int ROT_LANES = 8;  // threads sharing one row

// Apply one rotation operator (parity 0: pairs at even F index, 1: odd) of
// time index n to the rows of the tile.  Pairs crossing a row boundary have a
// zero angle in the reference (mesh_operators.py:996-999) and are skipped.
template <typename R>
__device__ __forceinline__ void rotate_rows(Cx<R>* tile, int rows, int nl, int j0, int jj, int lane,
                                            int parity, const RotTab<R>& tb, R tau, R efield) {
    if (jj < rows) {
        const int j = j0 + jj;
        const int l0 = int((int64_t(j) * nl + parity) & 1);
        const R rqj = tb.rq[j];
        for (int l = l0 + 2 * lane; l + 1 < nl; l += 2 * ROT_LANES) {
            const R theta = tau * ((tb.cl[l] * rqj) * efield);
            R s, c;
            sincos_r(theta, &s, &c);
            Cx<R>* p0 = tile + l * rows + jj;
            Cx<R>* p1 = p0 + rows;
            const Cx<R> x0 = *p0, x1 = *p1;
            *p0 = Cx<R>{c * x0.re + s * x1.im, c * x0.im - s * x1.re};
            *p1 = Cx<R>{s * x0.im + c * x1.re, c * x1.im - s * x0.re};
        }
    }
    __syncwarp();
}

// block-wide FP64 sum (result valid in thread 0)
__device__ __forceinline__ double block_sum(double v, double* scratch) {
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

// per-tile partial sums of |g|^2 and conj(s) g for every test state
template <typename R>
__device__ void reduce_tile(const ion_sh_sim& S, const Cx<R>* tile, int rows, int nl, int j0,
                            int tile_idx, double* scratch) {
    const int nq = 1 + 2 * S.n_states;
    const int jj = threadIdx.x / ROT_LANES, lane = threadIdx.x % ROT_LANES;
    // norm
    double acc = 0.0;
    if (jj < rows)
        for (int l = lane; l < nl; l += ROT_LANES) {
            const Cx<R> x = tile[l * rows + jj];
            acc += double(x.re) * double(x.re) + double(x.im) * double(x.im);
        }
    double tot = block_sum(acc, scratch);
    if (threadIdx.x == 0) S.partials[int64_t(tile_idx) * nq] = tot;
    // inner products with the test states: only row l_s of each state
    for (int s = 0; s < S.n_states; ++s) {
        const int ls = S.state_l[s];
        double re = 0.0, im = 0.0;
        if (lane == 0 && jj < rows && ls < nl) {
            const Cx<R> x = tile[ls * rows + jj];
            const double* sg = S.state_g + (int64_t(s) * S.n_r + j0 + jj) * 2;
            const double ar = sg[0], ai = -sg[1];  // conj(state)
            re = ar * double(x.re) - ai * double(x.im);
            im = ar * double(x.im) + ai * double(x.re);
        }
        const double tr = block_sum(re, scratch);
        const double ti = block_sum(im, scratch);
        if (threadIdx.x == 0) {
            S.partials[int64_t(tile_idx) * nq + 1 + 2 * s] = tr;
            S.partials[int64_t(tile_idx) * nq + 2 + 2 * s] = ti;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(256) sh_rot_kernel(ion_sh_plan plan, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int si = plan.rot_items[2 * blockIdx.x];
    const int tile_idx = plan.rot_items[2 * blockIdx.x + 1];
    const ion_sh_sim& S = plan.sims[si];
    const int64_t t = S.t;
    const int64_t tf = S.t_final;

    bool post = false, do_mask = false, reduce = false, pre = false;
    int64_t n_post = 0, n_pre = 0, t_reduce = 0;
    if (mode == ROT_PRE_ONLY) {
        if (t >= tf) return;
        pre = true;
        n_pre = t + 1;
    } else if (mode == ROT_STEP || mode == ROT_STEP_PRE) {
        if (t >= tf) return;
        post = true;
        n_post = t + 1;
        do_mask = S.mask != nullptr;
        reduce = is_data_time(t + 1, tf, S.store_every);
        t_reduce = t + 1;
        if (mode == ROT_STEP_PRE && t + 1 < tf) {
            pre = true;
            n_pre = t + 2;
        }
    } else if (mode == ROT_REDUCE_ONLY) {
        reduce = is_data_time(t, tf, S.store_every);
        t_reduce = t;
        if (!reduce) return;
    }
    (void)t_reduce;

    const int nr = S.n_r, nl = S.n_l;
    const int rows_max = plan.rot_rows;
    const int j0 = tile_idx * rows_max;
    const int rows = min(rows_max, nr - j0);
    if (rows <= 0) return;
    Cx<R>* tile = reinterpret_cast<Cx<R>*>(smem_raw);
    double* scratch = reinterpret_cast<double*>(tile + size_t(plan.max_n_l) * rows_max);
    Cx<R>* g = static_cast<Cx<R>*>(S.g);

    for (int f = threadIdx.x; f < nl * rows; f += blockDim.x) {
        const int l = f / rows, jj = f - l * rows;
        tile[l * rows + jj] = ld(g + int64_t(l) * nr + j0 + jj);
    }
    __syncthreads();

    const RotTab<R> tb = RotTab<R>::make(S);
    const int jj = threadIdx.x / ROT_LANES, lane = threadIdx.x % ROT_LANES;
    if (post) {
        const R tau = R(S.tau[n_post]), ef = R(S.efield[n_post]);
        rotate_rows<R>(tile, rows, nl, j0, jj, lane, 1, tb, tau, ef);  // odd
        rotate_rows<R>(tile, rows, nl, j0, jj, lane, 0, tb, tau, ef);  // even
    }
    if (do_mask && jj < rows) {
        const R mk = tb.mask[j0 + jj];
        for (int l = lane; l < nl; l += ROT_LANES) {
            Cx<R>* p = tile + l * rows + jj;
            *p = Cx<R>{p->re * mk, p->im * mk};
        }
    }
    __syncthreads();
    if (reduce) {
        reduce_tile<R>(S, tile, rows, nl, j0, tile_idx, scratch);
        __syncthreads();
    }
    if (pre) {
        const R tau = R(S.tau[n_pre]), ef = R(S.efield[n_pre]);
        rotate_rows<R>(tile, rows, nl, j0, jj, lane, 0, tb, tau, ef);  // even
        rotate_rows<R>(tile, rows, nl, j0, jj, lane, 1, tb, tau, ef);  // odd
    }
    __syncthreads();
    if (post || pre || do_mask) {
        for (int f = threadIdx.x; f < nl * rows; f += blockDim.x) {
            const int l = f / rows, jj2 = f - l * rows;
            st(g + int64_t(l) * nr + j0 + jj2, tile[l * rows + jj2]);
        }
    }
}

// Neumaier-compensated sum of the per-tile partials, then advance t
__global__ void sh_advance_kernel(ion_sh_plan plan, int mode) {
    ion_sh_sim& S = plan.sims[blockIdx.x];
    const int64_t t = S.t, tf = S.t_final;
    int64_t tr;
    if (mode == ADV_STEP) {
        if (t >= tf) return;
        tr = t + 1;
    } else {
        tr = t;
    }
    if (is_data_time(tr, tf, S.store_every)) {
        const int nq = 1 + 2 * S.n_states;
        const int64_t slot = data_slot(tr, tf, S.store_every);
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            double sum = 0.0, comp = 0.0;
            for (int k = 0; k < S.n_tiles; ++k) {
                const double v = S.partials[int64_t(k) * nq + q];
                const double tsum = sum + v;
                if (fabs(sum) >= fabs(v))
                    comp += (sum - tsum) + v;
                else
                    comp += (v - tsum) + sum;
                sum = tsum;
            }
            sum = (sum + comp) * S.weight;
            if (q == 0)
                S.out_norm[slot] = sum;
            else
                S.out_ip[(slot * S.n_states) * 2 + (q - 1)] = sum;
        }
    }
    __syncthreads();
    if (mode == ADV_STEP && threadIdx.x == 0) S.t = t + 1;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
template <typename R>
static int sh_validate(const ion_sh_plan* p) {
    if (!p || !p->sims || p->n_sims < 0 || p->n_cn_items < 0 || p->n_rot_items < 0 ||
        p->rot_rows <= 0 || p->rot_rows > 64 || p->max_n_l <= 0 || p->max_n_r < 2 ||
        p->cn_threads <= 0 || p->cn_threads > ShCfg<R>::MAX_T || (p->cn_threads & 31) ||
        int64_t(p->max_n_r) > int64_t(ShCfg<R>::MAXM) * ShCfg<R>::MAX_T) {
        set_error("ion_sh: invalid plan");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (sh_line_threads(p->max_n_r, ShCfg<R>::MAXM) > p->cn_threads) {
        set_error("ion_sh: cn_threads %d too small for n_r %d", p->cn_threads, p->max_n_r);
        return ION_ERR_INVALID_ARGUMENT;
    }
    return ION_OK;
}

template <typename R>
static size_t rot_smem(const ion_sh_plan* p) {
    return size_t(p->max_n_l) * p->rot_rows * sizeof(Cx<R>) + 32 * sizeof(double);
}

template <typename R>
static int sh_launch_rot(const ion_sh_plan* p, int mode, cudaStream_t s) {
    if (p->n_rot_items == 0) return ION_OK;
    const size_t smem = rot_smem<R>(p);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(sh_rot_kernel<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    sh_rot_kernel<R><<<p->n_rot_items, p->rot_rows * ROT_LANES, smem, s>>>(*p, mode);
    return check_launch("sh_rot_kernel");
}

template <typename R>
static int sh_launch_cn(const ion_sh_plan* p, cudaStream_t s) {
    if (p->n_cn_items == 0) return ION_OK;
    constexpr int MAXM = ShCfg<R>::MAXM;
    const size_t smem = sh_cn_smem<R>(p->max_n_r, p->cn_threads);
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(sh_cn_kernel<R, MAXM>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    if (smem > 200 * 1024) {
        set_error("ion_sh: radial line too long for shared memory");
        return ION_ERR_UNSUPPORTED;
    }
    sh_cn_kernel<R, MAXM><<<p->n_cn_items, p->cn_threads, smem, s>>>(*p);
    return check_launch("sh_cn_kernel");
}

template <typename R>
static int sh_run(const ion_sh_plan* p, int64_t n_steps, void* stream) {
    if (int e = sh_validate<R>(p)) return e;
    if (n_steps < 0) {
        set_error("ion_sh: negative step count");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (n_steps == 0 || p->n_sims == 0) return ION_OK;
    cudaStream_t s = as_stream(stream);
    if (int e = sh_launch_rot<R>(p, ROT_PRE_ONLY, s)) return e;
    for (int64_t k = 0; k < n_steps; ++k) {
        if (int e = sh_launch_cn<R>(p, s)) return e;
        if (int e = sh_launch_rot<R>(p, k + 1 < n_steps ? ROT_STEP_PRE : ROT_STEP, s)) return e;
        sh_advance_kernel<<<p->n_sims, 32, 0, s>>>(*p, ADV_STEP);
        if (int e = check_launch("sh_advance_kernel")) return e;
    }
    return ION_OK;
}

template <typename R>
static int sh_reduce(const ion_sh_plan* p, void* stream) {
    if (int e = sh_validate<R>(p)) return e;
    if (p->n_sims == 0) return ION_OK;
    cudaStream_t s = as_stream(stream);
    if (int e = sh_launch_rot<R>(p, ROT_REDUCE_ONLY, s)) return e;
    sh_advance_kernel<<<p->n_sims, 32, 0, s>>>(*p, ADV_FINALIZE);
    return check_launch("sh_advance_kernel");
}

}  // namespace ion

using namespace ion;

extern "C" {

int ion_sh_split_run_c128(const ion_sh_plan* plan, int64_t n_steps, void* stream) {
    return sh_run<double>(plan, n_steps, stream);
}
int ion_sh_split_run_c64(const ion_sh_plan* plan, int64_t n_steps, void* stream) {
    return sh_run<float>(plan, n_steps, stream);
}
int ion_sh_reduce_c128(const ion_sh_plan* plan, void* stream) { return sh_reduce<double>(plan, stream); }
int ion_sh_reduce_c64(const ion_sh_plan* plan, void* stream) { return sh_reduce<float>(plan, stream); }
int64_t ion_sh_max_n_r_c128(void) { return int64_t(ShCfg<double>::MAXM) * ShCfg<double>::MAX_T; }
int64_t ion_sh_max_n_r_c64(void) { return int64_t(ShCfg<float>::MAXM) * ShCfg<float>::MAX_T; }

}  // extern "C"
