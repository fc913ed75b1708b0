// Spherical-harmonic (l, r) mesh, length gauge, split-interaction operator.
//
// Reference path: SplitInteractionOperator.get_evolution_operators
// (ionization/mesh/evolution_methods.py:89-123) over
// SphericalHarmonicLengthGaugeOperators (ionization/mesh/mesh_operators.py:
// 815-1080), applied by QuantumMesh.evolve (ionization/mesh/meshes.py:251-257)
// once per step of MeshSimulation.run (ionization/mesh/sims.py:289-333).
//
// Per step three kinds of kernel run on the whole batch:
//   sh_cn_pipelined  the radial solves, one launch per bucket of lines of
//                  similar length (each with its own CTA size and rows per
//                  thread): persistent CTAs, each walking the
//                  (simulation, l) lines of its bucket with
//                  the next line's psi streaming into shared memory while the
//                  current one is solved; y = (1 - i tau H0) psi is formed on
//                  the fly and (1 + i tau H0) x = y is solved by the block
//                  partition + PCR solver;
//   sh_rot_kernel  one CTA per (simulation, tile of r rows) holding all l of
//                  those rows: the rotations after the radial solve of step
//                  t+1 (odd, even), the mask, the data-time reductions, and
//                  the rotations before the radial solve of step t+2 (even,
//                  odd), all fused in one pass;
//   sh_advance_kernel  finishes the reductions (compensated sum over tiles)
//                  and advances each simulation's time index.
#include <cstdio>

#include <algorithm>

#include "ion_common.cuh"
#include <type_traits>

#include "ion_cn_solver.cuh"

namespace ion {

enum : int { ROT_PRE_ONLY = 1, ROT_STEP = 2, ROT_STEP_PRE = 3, ROT_REDUCE_ONLY = 4 };
enum : int { ADV_STEP = 1, ADV_FINALIZE = 2 };

constexpr int ROT_LANES = 8;  // threads sharing one row of a rotation tile
constexpr int ROT_ROWS = 32;  // r rows per rotation tile (the shared-memory stride)

template <typename R> struct ShCfg;
template <> struct ShCfg<double> {
    static constexpr int MAXM = 8;
    static constexpr int MAX_T = 512;
};
template <> struct ShCfg<float> {
    static constexpr int MAXM = 16;
    static constexpr int MAX_T = 512;
};

// threads of the radial solve of a line of nr points: nr rounded up to
// whole chunks of maxm rows
__host__ __device__ inline int sh_line_threads(int nr, int maxm) { return (nr + maxm - 1) / maxm; }

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

// A = 1 + i tau H0 on line l: coefficients for the CN solver (tau-scaled)
template <typename R>
struct ShCnCoef {
    ShH<R> h;
    R tau;
    int n;
    __device__ __forceinline__ void operator()(int i, R& bo, R& bd) const {
        if (i >= n) {
            bo = R(0);
            bd = R(0);
            return;
        }
        bd = tau * h.diag(i);
        bo = (i < n - 1) ? tau * h.off(i) : R(0);
    }
};

// psi + delta into the interleaved line
template <typename R, int M>
struct AddOut {
    Cx<R>* line;
    int T;
    __device__ __forceinline__ void operator()(int i, Cx<R> d) const {
        Cx<R>* p = line + islot<M>(i, T);
        *p = *p + d;
    }
};

// psi + delta, or delta alone (``add`` false), into the interleaved line
template <typename R, int M>
struct AddOrSetOut {
    Cx<R>* line;
    int T;
    bool add;
    __device__ __forceinline__ void operator()(int i, Cx<R> d) const {
        Cx<R>* p = line + islot<M>(i, T);
        *p = add ? *p + d : d;
    }
};

// (h + d) with the residual lo: h + d is formed exactly (Knuth's TwoSum), its
// rounding error joins lo, and the pair is renormalised (Fast2Sum).  Returns
// the new h; lo is updated in place.
template <typename R>
__device__ __forceinline__ R add_exact1(R h, R d, R& lo) {
    const R s = h + d;
    const R bb = s - h;
    const R e = (h - (s - bb)) + (d - bb);
    const R l = lo + e;
    const R r = s + l;
    lo = l - (r - s);
    return r;
}
template <typename R>
__device__ __forceinline__ Cx<R> add_exact(Cx<R> h, Cx<R> d, Cx<R>& lo) {
    return Cx<R>{add_exact1(h.re, d.re, lo.re), add_exact1(h.im, d.im, lo.im)};
}

__device__ __forceinline__ void prefetch_l2(const void* p) {
    asm volatile("prefetch.global.L2 [%0];\n" ::"l"(p));
}

// L2 prefetch of the rows of rotation tile ``item`` (n_l segments of
// ROT_ROWS points)
template <typename R>
__device__ __forceinline__ void prefetch_rot_item(const ion_sh_plan& plan, int item) {
    const int si = plan.rot_items[2 * item];
    const int tile = plan.rot_items[2 * item + 1];
    const ion_sh_sim& S = plan.sims[si];
    const Cx<R>* g = static_cast<const Cx<R>*>(S.g);
    constexpr int per_seg = (32 * int(sizeof(Cx<R>)) + 127) / 128;  // cache lines per l segment
    for (int f = threadIdx.x; f < S.n_l * per_seg; f += blockDim.x) {
        const int l = f / per_seg, c = f - l * per_seg;
        const char* p = reinterpret_cast<const char*>(g + int64_t(l) * S.n_r + tile * 32) + c * 128;
        prefetch_l2(p);
    }
}

// ---------------------------------------------------------------------------
// Pipelined radial solve: a persistent CTA walks the items of one bucket
// (item0 + blockIdx.x, then every gridDim.x-th).  While it solves one line,
// the psi of its next line is already streaming into the other of two
// shared-memory buffers (cp.async, no registers held), so the global-load
// latency of the staging overlaps the solve instead of stalling it.  The
// coefficients are formed in the chunk elimination from the per-r tables,
// which every line of a simulation shares (they stay in L1); the complex64
// tables are padded with zeros to a multiple of 16 entries, so a chunk of
// M = 8 or 16 rows is read with 16-byte vector loads.
// ---------------------------------------------------------------------------
// RES: the explicit half is formed in the residual form below (with a stored
// residual ``lo``, which may still be NULL); otherwise plainly.
template <bool RES>
struct ShCnCoef32 {
    const float* kinv;
    const float* cent;
    const float* hoff;
    float ll1, corr0, tau;
    int n;
    // the line's stored residual (c64x, packed bf16x2) staged in shared memory
    // in the line's interleaved layout (slot (i mod 2^mshift) T + i >> mshift),
    // or NULL
    const uint32_t* lob;
    int T, mshift;
    // the line's row-sum remainders (ion_sh_sim.row_lo, bf16) staged in
    // shared memory in row order, or NULL: with them the explicit half
    // applies the FP64 Hamiltonian (the refinement)
    const uint16_t* rlo;
    __device__ __forceinline__ Cx<float> lo_at(int i) const {
        return lo_unpack(lob[(i & ((1 << mshift) - 1)) * T + (i >> mshift)]);
    }
    __device__ __forceinline__ float row_rem(int i) const { return __uint_as_float(uint32_t(rlo[i]) << 16); }
    // the FP32 diagonal before tau, as every solve forms it (load_chunk too)
    __device__ __forceinline__ void operator()(int i, float& bo, float& bd) const {
        if (i < 0 || i >= n) {
            bo = 0.f;
            bd = 0.f;
            return;
        }
        float h = fmaf(ll1, cent[i], kinv[i]);
        if (i == 0) h = h + corr0;
        bd = tau * h;
        bo = (i < n - 1) ? tau * hoff[i] : 0.f;
    }
};

template <int M, bool RES>
__device__ __forceinline__ void load_chunk(const ShCnCoef32<RES>& c, int s, float (&bo)[M], float (&bd)[M]) {
    static_assert(M % 4 == 0, "whole float4 groups");
#pragma unroll
    for (int q = 0; q < M / 4; ++q) {
        const float4 kv = __ldg(reinterpret_cast<const float4*>(c.kinv + s) + q);
        const float4 cv = __ldg(reinterpret_cast<const float4*>(c.cent + s) + q);
        const float4 hv = __ldg(reinterpret_cast<const float4*>(c.hoff + s) + q);
        const float kk[4] = {kv.x, kv.y, kv.z, kv.w}, cc[4] = {cv.x, cv.y, cv.z, cv.w},
                    hh[4] = {hv.x, hv.y, hv.z, hv.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int k = 4 * q + e, i = s + k;
            float h = fmaf(c.ll1, cc[e], kk[e]);  // as ShCnCoef32::operator()
            if (i == 0) h = h + c.corr0;
            bd[k] = i < c.n ? c.tau * h : 0.f;
            bo[k] = i < c.n - 1 ? c.tau * hh[e] : 0.f;
        }
    }
}

// The explicit half-step of the complex64 radial solve, with a stored residual.
// Its kinetic terms are ~1/dr^2 times psi and cancel to ~E psi, so forming
// a0 psi_{i-1} + bd psi_i + bo psi_{i+1} in FP32 leaves a random error of
// ~1e-8 |psi| per step, which once the state's own rounding is gone is the
// dominant error over 10^4 steps.  The same FP32 coefficients are used as
//   a0 (psi_{i-1} - psi_i) + bo (psi_{i+1} - psi_i) + (a0 + bd + bo) psi_i,
// with the row sum a0 + bd + bo formed exactly as a two-float (TwoSum), so
// the explicit operator equals the implicit one exactly (the step stays
// unitary) and no product is of a large, cancelling quantity.
__device__ __forceinline__ float two_sum_err(float a, float b, float& e) {
    const float s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
    return s;
}

// The residual itself enters B psi as well: most of a step's sub-ulp
// increment is what lands in the residual, so leaving B lo out of the right
// side would bias every step the same way (a steady norm drift).  B lo is
// tiny and formed plainly.
template <bool RES>
__device__ __forceinline__ Cx<float> stencil_row(const ShCnCoef32<RES>& c, int i, float a0, float bd, float bo,
                                                  Cx<float> p0, Cx<float> p1, Cx<float> p2) {
    if (!RES || c.lob == nullptr)
        return Cx<float>{a0 * p0.re + bd * p1.re + bo * p2.re, a0 * p0.im + bd * p1.im + bo * p2.im};
    float e1, e2;
    const float s1 = two_sum_err(bd, a0, e1);
    const float rs = two_sum_err(s1, bo, e2);
    float rl = e1 + e2;  // rs + rl = a0 + bd + bo to ~2^-48
    // with the remainders, rs + rl is the FP64 Hamiltonian's row sum; the
    // couplings' own roundings act on neighbour differences only, which
    // matters far less (a relative error of ~1e-7 in the kinetic energy)
    if (c.rlo != nullptr && i < c.n) rl += c.row_rem(i);
    const Cx<float> dm = p0 - p1, dp = p2 - p1;
    Cx<float> v = {a0 * dm.re + bo * dp.re + (rs * p1.re + rl * p1.re),
                   a0 * dm.im + bo * dp.im + (rs * p1.im + rl * p1.im)};
    if (i < c.n) {  // padding rows carry no residual
        const Cx<float> l1 = c.lo_at(i);
        const Cx<float> l0 = i > 0 ? c.lo_at(i - 1) : Cx<float>{0.f, 0.f};
        const Cx<float> l2 = i + 1 < c.n ? c.lo_at(i + 1) : Cx<float>{0.f, 0.f};
        v.re += a0 * l0.re + bd * l1.re + bo * l2.re;
        v.im += a0 * l0.im + bd * l1.im + bo * l2.im;
    }
    return v;
}

template <typename R, bool RES> struct ShCnCoefFor;
template <bool RES> struct ShCnCoefFor<double, RES> {
    using type = ShCnCoef<double>;
    __device__ static type make(const ion_sh_sim& S, int l, double tau, const void*, int, int,
                                const uint16_t* = nullptr) {
        return type{ShH<double>::make(S, l), tau, S.n_r};
    }
};
template <bool RES> struct ShCnCoefFor<float, RES> {
    using type = ShCnCoef32<RES>;
    // lob: the line's residual staged in shared memory, or NULL; rlo: its
    // row-sum remainders staged in shared memory (row i at rlo[i]), or NULL
    __device__ static type make(const ion_sh_sim& S, int l, float tau, const void* lob, int T, int mshift,
                                const uint16_t* rlo = nullptr) {
        return type{S.kinv32, S.cent32, S.hoff32, float(l) * float(l + 1), (l == 0) ? S.corr0_32 : 0.f, tau, S.n_r,
                    static_cast<const uint32_t*>(lob), T, mshift, rlo};
    }
};

// The row-sum remainders of line l (bf16, row_lo + l n_r, any 2-byte
// alignment) into ``dst`` (16-byte aligned, sh_rlo_words(cap) halfwords) by
// 16-byte asynchronous copies of the aligned blocks that cover the line: row i
// lands at dst[rlo_shift(src) + i].  A block that would reach outside the
// array [row_lo, row_lo + n_l n_r) is copied by element, zero outside.
__device__ __forceinline__ int rlo_shift(const uint16_t* src) {
    return int((reinterpret_cast<uintptr_t>(src) & 15u) >> 1);
}
__device__ __forceinline__ void stage_row_lo(const ion_sh_sim& S, int l, uint16_t* dst) {
    const int nr = S.n_r;
    const uint16_t* src = S.row_lo + int64_t(l) * nr;
    const uint16_t* base = src - rlo_shift(src);
    const uint16_t* lo_end = S.row_lo + int64_t(S.n_l) * nr;
    const int nblk = (rlo_shift(src) + nr + 7) >> 3;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        const uint16_t* p = base + 8 * b;
        if (p >= S.row_lo && p + 8 <= lo_end) {
            cp_async16(dst + 8 * b, p);
        } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) dst[8 * b + e] = (p + e >= S.row_lo && p + e < lo_end) ? p[e] : uint16_t(0);
        }
    }
}

// halfwords of one staged row_lo buffer for lines of up to ``cap`` rows
__host__ __device__ inline int sh_rlo_words(int cap) { return (cap + 8 + 7) / 8 * 8; }

// psi of item ``item`` into ``dst`` (interleaved, zero padding), its stored
// residual (packed bf16x2) into ``lodst`` and its row-sum remainders into
// ``rlodst`` when given (complex64 with g_lo), asynchronously
template <typename R, int M>
__device__ __forceinline__ void sh_cn_stage_async(const ion_sh_plan& plan, int item, Cx<R>* dst,
                                                  uint32_t* lodst = nullptr, uint16_t* rlodst = nullptr) {
    const int si = plan.cn_items[2 * item];
    const int l = plan.cn_items[2 * item + 1];
    const ion_sh_sim& S = plan.sims[si];
    if (S.t >= S.t_final) return;
    const int nr = S.n_r;
    const int T = (nr + M - 1) / M;
    if (T > int(blockDim.x)) return;  // a line longer than the CTA holds: skipped (see below)
    const int npad = T * M;
    const Cx<R>* g = static_cast<const Cx<R>*>(S.g) + int64_t(l) * nr;
    const uint32_t* glo = (lodst && S.g_lo) ? static_cast<const uint32_t*>(S.g_lo) + int64_t(l) * nr : nullptr;
    if (glo && rlodst && S.row_lo) stage_row_lo(S, l, rlodst);
    for (int i = threadIdx.x; i < npad; i += blockDim.x) {
        Cx<R>* d = dst + islot<M>(i, T);
        if (i < nr) {
            if (sizeof(Cx<R>) == 16)
                cp_async16(d, g + i);
            else
                cp_async8(d, g + i);
            if (glo) cp_async4(lodst + islot<M>(i, T), glo + i);
        } else {
            *d = Cx<R>{R(0), R(0)};
            if (glo) lodst[islot<M>(i, T)] = 0u;
        }
    }
}

// X_i = -i d_i with d read from an interleaved line buffer, or 0 (``on`` false)
template <typename R, int M>
struct MinusIExtra {
    const Cx<R>* d;
    int T;
    bool on;
    template <typename RR>
    __device__ __forceinline__ Cx<RR> get(int i) const {
        if (!on) return Cx<RR>{RR(0), RR(0)};
        const Cx<R> v = d[islot<M>(i, T)];
        return Cx<RR>{v.im, -v.re};
    }
};

// ``dbuf`` 0: one line buffer (lines too long for two), staged at the top of
// each iteration without overlap.  ``refine`` 1: a third line buffer holds the
// increment, and the simulations with a stored residual refine their solve:
// with Delta1 from A Delta1 = Y, the correction solves
//   A delta = Y - A Delta1 = -i B (2 psi + Delta1) - Delta1,
// i.e. the same solver on phi = psi + Delta1 / 2 with X = -i Delta1, so the
// fixed rounding of the elimination of A acts only on the small residual.
// 4 rows per thread (complex64) fits in 64 registers, so those CTAs may
// hold up to 1024 threads (lines of up to 4096 points at 32 warps an SM)
template <typename R, int M>
__host__ __device__ constexpr int sh_cn_max_threads() {
    return (M == 4 && sizeof(R) == 4) ? 1024 : 512;
}

template <typename R, int M, bool REFINE>
__global__ void __launch_bounds__(sh_cn_max_threads<R, M>()) sh_cn_pipelined(ion_sh_plan plan, int item0, int item_end, int dbuf) {
    constexpr int refine = REFINE ? 1 : 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int cap = blockDim.x * M;
    // psi (double-buffered), with refinement the increment, the staged
    // residual (packed) and row-sum remainders (both double-buffered like
    // psi), then the PCR scratch
    const int nb = dbuf ? 2 : 1;
    Cx<R>* buf0 = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* buf1 = buf0 + cap;
    Cx<R>* ext = buf0 + nb * cap;
    uint32_t* lob0 = reinterpret_cast<uint32_t*>(ext + (refine ? cap : 0));
    uint32_t* lob1 = lob0 + (dbuf ? cap : 0);
    uint16_t* rlo0 = reinterpret_cast<uint16_t*>(lob0 + (refine ? nb * cap : 0));
    uint16_t* rlo1 = rlo0 + (dbuf ? sh_rlo_words(cap) : 0);
    Cx<R>* red = reinterpret_cast<Cx<R>*>(rlo0 + (refine ? nb * sh_rlo_words(cap) : 0));
    int item = item0 + blockIdx.x;
    if (item >= item_end) return;
    if (dbuf) {
        sh_cn_stage_async<R, M>(plan, item, buf0, refine ? lob0 : nullptr, refine ? rlo0 : nullptr);
        cp_async_commit();
    }
    for (int j = 0; item < item_end; item += gridDim.x, ++j) {
        Cx<R>* cur = (dbuf && (j & 1)) ? buf1 : buf0;
        uint32_t* lob = (dbuf && (j & 1)) ? lob1 : lob0;
        uint16_t* rlo = (dbuf && (j & 1)) ? rlo1 : rlo0;
        if (dbuf) {
            const int next = item + gridDim.x;
            if (next < item_end)
                sh_cn_stage_async<R, M>(plan, next, (j & 1) ? buf0 : buf1, refine ? ((j & 1) ? lob0 : lob1) : nullptr,
                                        refine ? ((j & 1) ? rlo0 : rlo1) : nullptr);
            cp_async_commit();
            cp_async_wait<1>();  // this item's psi has landed; the next one stays in flight
        } else {
            sh_cn_stage_async<R, M>(plan, item, buf0, refine ? lob0 : nullptr, refine ? rlo0 : nullptr);
            cp_async_commit();
            cp_async_wait<0>();
        }
        __syncthreads();
        const int si = plan.cn_items[2 * item];
        const int l = plan.cn_items[2 * item + 1];
        const ion_sh_sim& S = plan.sims[si];
        const int64_t t = S.t;
        // a line the CTA cannot hold (a plan whose bucket does not fit its
        // lines) is left as it is rather than written out of bounds
        if (t < S.t_final && (S.n_r + M - 1) / M <= int(blockDim.x)) {  // the same for every thread of the CTA
            const int nr = S.n_r;
            const int T = (nr + M - 1) / M;
            const R tau = R(S.tau[t + 1]);
            // with a stored residual the solve leaves the increment in ``inc``
            uint32_t* glo = sizeof(R) == 4 && S.g_lo ? static_cast<uint32_t*>(S.g_lo) + int64_t(l) * nr : nullptr;
            const int mshift = M == 16 ? 4 : (M == 8 ? 3 : 2);
            // With refinement the first solve needs only an approximation of
            // delta1: the second forms the exact residual of whatever delta1
            // is and leaves (I - A'^-1 A) times its error, ~1e-4 of it (the
            // second solve's own PCR stops at 2^-13), so the first uses the
            // plain FP32 stencil, without the exact row sums and the residual
            // terms (an error of ~1e-5 of delta1, ~1e-9 after the correction).
            const auto coef = ShCnCoefFor<R, REFINE>::make(S, l, tau, nullptr, T, mshift);
            Cx<R>* inc = cur;
            if constexpr (REFINE) {
                // two solves through one call site: delta1 into ext, then on
                // phi = psi + delta1 / 2 (formed as it is read, so cur keeps
                // psi for the store) delta1 + delta into ext.  The second
                // forms its residual with the FP64 Hamiltonian's row sums
                // (ion_sh_sim.row_lo), so the refined solve converges to the
                // FP64 system.
                const bool two = glo != nullptr;
                if (two) inc = ext;
                const uint16_t* rl =
                    (refine && glo && S.row_lo) ? rlo + rlo_shift(S.row_lo + int64_t(l) * nr) : nullptr;
                const auto coef2 = ShCnCoefFor<R, REFINE>::make(S, l, tau, (refine && glo) ? lob : nullptr, T,
                                                                mshift, rl);
                for (int pass = 0; pass < (two ? 2 : 1); ++pass) {
                    // The correction of the second solve is ~1e-7 of delta1,
                    // so its reduced system may stop at couplings below
                    // 2^-13: the error left, ~1e-4 of the correction, is far
                    // below the FP32 rounding of the coefficients.
                    block_cn_solve<R, M>(T, threadIdx.x, R(2), HalfStepView<R>{cur, ext, pass == 1}, red,
                                         pass == 1 ? coef2 : coef,
                                         MinusIExtra<R, M>{ext, T, pass == 1},
                                         AddOrSetOut<R, M>{inc, T, pass == 1 || !two},
                                         pass == 1 ? R(1.0 / 8192.0) : PcrTiny<R>::value);
                    __syncthreads();
                }
            } else {
                // plain: psi + delta into cur; with a residual: delta into cur
                block_cn_solve<R, M>(T, threadIdx.x, R(2), cur, red, coef, NoExtra{},
                                     AddOrSetOut<R, M>{cur, T, glo == nullptr});
                __syncthreads();
            }
            Cx<R>* g = static_cast<Cx<R>*>(S.g) + int64_t(l) * nr;
            if (glo) {
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    const int i = threadIdx.x + k * blockDim.x;
                    if (i < nr) {
                        // refined: cur still holds psi; otherwise the increment
                        const Cx<float> lo0 = lo_unpack(refine ? lob[islot<M>(i, T)] : glo[i]);
                        Cx<R> lo = Cx<R>{R(lo0.re), R(lo0.im)};
                        const Cx<R> h = add_exact(refine ? cur[islot<M>(i, T)] : ld(g + i), inc[islot<M>(i, T)], lo);
                        st(g + i, h);
                        glo[i] = lo_pack(Cx<float>{float(lo.re), float(lo.im)});
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < M; ++k) {
                    const int i = threadIdx.x + k * blockDim.x;
                    if (i < nr) st(g + i, cur[islot<M>(i, T)]);
                }
            }
        }
        __syncthreads();  // every read of ``cur`` is done before it is refilled
    }
    cp_async_wait<0>();
}

// psi (x2 when double-buffered); with refinement the increment, the packed
// residual (4 bytes a row) and the row-sum remainders (2 bytes a row, 16-byte
// blocks), both x2 when double-buffered; the PCR scratch
template <typename R>
__host__ __device__ inline size_t sh_cn_pipelined_smem(int threads, int M, int refine, int dbuf) {
    const size_t cap = size_t(threads) * M;
    const size_t nb = dbuf ? 2 : 1;
    return nb * cap * sizeof(Cx<R>) +
           (refine ? cap * sizeof(Cx<R>) + nb * cap * 4 + nb * size_t(sh_rlo_words(int(cap))) * 2 : 0) +
           pcr_cn_smem_bytes<R>(threads);
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

// Dekker's Fast2Sum: a + b = s + e exactly when |a| >= |b|, which holds for
// the small rotation increments added to psi here
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
    const float s = a + b;
    e = b - (s - a);
    return s;
}

// The tile holds psi as hi (+ lo for complex64: a compensation word that
// collects the rounding of every update inside the pass, folded in once
// when psi is stored).  The rotation and the mask are written once, on
// register values, with every product-add an explicit fma: a launch that
// chains several operators on one pair in registers does exactly the
// arithmetic of one that goes through shared memory between them, so the
// result does not depend on how steps are split into launches.
template <typename R> struct Tile;
template <> struct Tile<double> {
    Cx<double>* hi;
    static constexpr bool comp = false;
    struct Pair {
        Cx<double> x0, x1;
    };
    __device__ Cx<double> value(int k) const { return hi[k]; }
    __device__ __forceinline__ Pair load(int k0, int k1) const { return Pair{hi[k0], hi[k1]}; }
    __device__ __forceinline__ void put(int k0, int k1, const Pair& p) const {
        hi[k0] = p.x0;
        hi[k1] = p.x1;
    }
    __device__ __forceinline__ static void rot(Pair& p, double cm1, double s) {
        const Cx<double> x0 = p.x0, x1 = p.x1;
        p.x0 = Cx<double>{x0.re + fma(cm1, x0.re, s * x1.im), x0.im + fma(cm1, x0.im, -(s * x1.re))};
        p.x1 = Cx<double>{x1.re + fma(cm1, x1.re, s * x0.im), x1.im + fma(cm1, x1.im, -(s * x0.re))};
    }
    __device__ __forceinline__ static Cx<double> scaled(Cx<double> h, double m) { return Cx<double>{h.re * m, h.im * m}; }
    __device__ __forceinline__ static void scale(Pair& p, double m) {
        p.x0 = scaled(p.x0, m);
        p.x1 = scaled(p.x1, m);
    }
    __device__ void rotate(int k0, int k1, double cm1, double s) const {
        Pair p = load(k0, k1);
        rot(p, cm1, s);
        put(k0, k1, p);
    }
    // velocity gauge: [[cos, sin], [-sin, cos]] in increment form
    __device__ void rotate_real(int k0, int k1, double cm1, double s) const {
        const Cx<double> x0 = hi[k0], x1 = hi[k1];
        hi[k0] = Cx<double>{x0.re + (cm1 * x0.re + s * x1.re), x0.im + (cm1 * x0.im + s * x1.im)};
        hi[k1] = Cx<double>{x1.re + (cm1 * x1.re - s * x0.re), x1.im + (cm1 * x1.im - s * x0.im)};
    }
    __device__ void scale(int k, double m) const { hi[k] = scaled(hi[k], m); }
    __device__ __forceinline__ static void renorm(Pair&, bool) {}
    __device__ void renorm(int, bool) const {}
    __device__ __forceinline__ static void quant(Pair&) {}
    __device__ Cx<double> out(int k) const { return hi[k]; }
    __device__ __forceinline__ void store(int k, Cx<double>* g, uint32_t*, int64_t at) const { st(g + at, hi[k]); }
};
// The complex64 tile keeps its compensation word lo packed as bf16x2, the
// format of the stored residual: every operator unpacks it, works in FP32 and
// packs it again, which is exactly what a store and a reload between two
// launches do to it, so results do not depend on where a run is cut into
// launches; the register sweeps that chain operators round lo the same way
// between them (``quant``).
template <> struct Tile<float> {
    Cx<float>* hi;
    uint32_t* lo;
    static constexpr bool comp = true;
    struct Pair {
        Cx<float> x0, x1, l0, l1;
    };
    __device__ Cx<double> value(int k) const {
        const Cx<float> l = lo_unpack(lo[k]);
        return Cx<double>{double(hi[k].re) + double(l.re), double(hi[k].im) + double(l.im)};
    }
    __device__ __forceinline__ Pair load(int k0, int k1) const {
        return Pair{hi[k0], hi[k1], lo_unpack(lo[k0]), lo_unpack(lo[k1])};
    }
    __device__ __forceinline__ void put(int k0, int k1, const Pair& p) const {
        hi[k0] = p.x0;
        hi[k1] = p.x1;
        lo[k0] = lo_pack(p.l0);
        lo[k1] = lo_pack(p.l1);
    }
    // lo as a put and a load between two operators leave it
    __device__ __forceinline__ static void quant(Pair& p) {
        p.l0 = lo_round(p.l0);
        p.l1 = lo_round(p.l1);
    }
    // x -> x + (cm1 x - i s y) for each element x of the pair and its partner
    // y, the sum exact through Fast2Sum with its error into lo.  Both
    // components go through one packed FP32 instruction each (FFMA2 / FADD2 /
    // FMUL2, per-component IEEE rounding, so the result is that of the scalar
    // form: x.re + fma(cm1, x.re, s y.im), x.im + fma(cm1, x.im, -(s y.re))).
    __device__ __forceinline__ static void rot1(Cx<float>& x, Cx<float>& l, Cx<float> y, Cx<float> ly, float2 c2,
                                                float2 s2) {
        const float2 X = make_float2(x.re, x.im), L = make_float2(l.re, l.im);
        const float2 u = __ffma2_rn(c2, X, __fmul2_rn(s2, make_float2(y.im, y.re)));
        const float2 h = __fadd2_rn(X, u);
        const float2 d = __fadd2_rn(h, make_float2(-X.x, -X.y));
        const float2 e = __fadd2_rn(u, make_float2(-d.x, -d.y));  // u - (h - x)
        const float2 v = __ffma2_rn(c2, L, __fmul2_rn(s2, make_float2(ly.im, ly.re)));
        const float2 ln = __fadd2_rn(__fadd2_rn(L, v), e);
        x = Cx<float>{h.x, h.y};
        l = Cx<float>{ln.x, ln.y};
    }
    __device__ __forceinline__ static void rot(Pair& p, float cm1, float s) {
        const Cx<float> x0 = p.x0, x1 = p.x1, l0 = p.l0, l1 = p.l1;
        const float2 c2 = make_float2(cm1, cm1), s2 = make_float2(s, -s);
        rot1(p.x0, p.l0, x1, l1, c2, s2);
        rot1(p.x1, p.l1, x0, l0, c2, s2);
    }
    // the product's rounding error goes to lo (packed: the scalar form
    // pr = h.re m, lo.re = fma(lo.re, m, fma(h.re, m, -pr)) per component)
    __device__ __forceinline__ static void scaled(Cx<float>& h, Cx<float>& l, float m) {
        const float2 M = make_float2(m, m), H = make_float2(h.re, h.im);
        const float2 P = __fmul2_rn(H, M);
        const float2 Ln = __ffma2_rn(make_float2(l.re, l.im), M, __ffma2_rn(H, M, make_float2(-P.x, -P.y)));
        l = Cx<float>{Ln.x, Ln.y};
        h = Cx<float>{P.x, P.y};
    }
    __device__ __forceinline__ static void scale(Pair& p, float m) {
        scaled(p.x0, p.l0, m);
        scaled(p.x1, p.l1, m);
    }
    __device__ void rotate(int k0, int k1, float cm1, float s) const {
        Pair p = load(k0, k1);
        rot(p, cm1, s);
        put(k0, k1, p);
    }
    __device__ void rotate_real(int k0, int k1, float cm1, float s) const {
        const Cx<float> x0 = hi[k0], x1 = hi[k1], l0 = lo_unpack(lo[k0]), l1 = lo_unpack(lo[k1]);
        float e0r, e0i, e1r, e1i;
        const float h0r = two_sum(x0.re, cm1 * x0.re + s * x1.re, e0r);
        const float h0i = two_sum(x0.im, cm1 * x0.im + s * x1.im, e0i);
        const float h1r = two_sum(x1.re, cm1 * x1.re - s * x0.re, e1r);
        const float h1i = two_sum(x1.im, cm1 * x1.im - s * x0.im, e1i);
        hi[k0] = Cx<float>{h0r, h0i};
        hi[k1] = Cx<float>{h1r, h1i};
        lo[k0] = lo_pack(Cx<float>{l0.re + (cm1 * l0.re + s * l1.re) + e0r, l0.im + (cm1 * l0.im + s * l1.im) + e0i});
        lo[k1] = lo_pack(Cx<float>{l1.re + (cm1 * l1.re - s * l0.re) + e1r, l1.im + (cm1 * l1.im - s * l0.im) + e1i});
    }
    __device__ void scale(int k, float m) const {
        Cx<float> h = hi[k], l = lo_unpack(lo[k]);
        scaled(h, l, m);
        hi[k] = h;
        lo[k] = lo_pack(l);
    }
    // what a store and a reload between launches do to (hi, lo): hi + lo
    // rounded, and with a stored residual (keep) its rounding error as lo
    // (Fast2Sum), else lo = 0
    __device__ __forceinline__ static void renorm(Cx<float>& h, Cx<float>& l, bool keep) {
        const float2 H = make_float2(h.re, h.im), L = make_float2(l.re, l.im);
        const float2 S = __fadd2_rn(H, L);
        const float2 D = __fadd2_rn(S, make_float2(-H.x, -H.y));
        const float2 E = __fadd2_rn(L, make_float2(-D.x, -D.y));  // l - (s - h)
        l = keep ? Cx<float>{E.x, E.y} : Cx<float>{0.f, 0.f};
        h = Cx<float>{S.x, S.y};
    }
    __device__ __forceinline__ static void renorm(Pair& p, bool keep) {
        renorm(p.x0, p.l0, keep);
        renorm(p.x1, p.l1, keep);
    }
    __device__ void renorm(int k, bool keep) const {
        Cx<float> h = hi[k], l = lo_unpack(lo[k]);
        renorm(h, l, keep);
        hi[k] = h;
        lo[k] = lo_pack(l);
    }
    __device__ Cx<float> out(int k) const {
        const Cx<float> l = lo_unpack(lo[k]);
        return Cx<float>{hi[k].re + l.re, hi[k].im + l.im};
    }
    // element k to g[at]: hi + lo folded, or, with a stored residual, hi + lo
    // renormalised (Fast2Sum, |hi| >= |lo|) into g[at] and glo[at] (packed)
    __device__ __forceinline__ void store(int k, Cx<float>* g, uint32_t* glo, int64_t at) const {
        const Cx<float> h = hi[k], l = lo_unpack(lo[k]);
        const float sr = h.re + l.re, si = h.im + l.im;
        st(g + at, Cx<float>{sr, si});
        if (glo) glo[at] = lo_pack(Cx<float>{l.re - (sr - h.re), l.im - (si - h.im)});
    }
};

// One rotation operator (parity 0: pairs at even F index, 1: odd) of time
// index n on every row of the tile.  Pairs crossing a row boundary have a
// zero angle in the reference (mesh_operators.py:996-999) and are skipped.
// Thread (jj, lane): jj = row of the tile, lane strides over the pairs.
template <typename R>
__device__ __forceinline__ void rotate_rows(const Tile<R>& tl, int rows, int nl, int j0, int jj, int lane, int lanes,
                                            int parity, const RotTab<R>& tb, R tau, R efield) {
    if (jj < rows) {
        const int j = j0 + jj;
        const int l0 = int((int64_t(j) * nl + parity) & 1);
        const R rqj = tb.rq[j];
        for (int l = l0 + 2 * lane; l + 1 < nl; l += 2 * lanes) {
            R cm1, s;
            rot_coeffs(tau * ((tb.cl[l] * rqj) * efield), cm1, s);
            tl.rotate(l * ROT_ROWS + jj, (l + 1) * ROT_ROWS + jj, cm1, s);
        }
    }
    __syncthreads();
}

// Between two solves with no data stored in between: the even rotation of
// time index n1, the mask, the renormalisation of (hi, lo) that a store and
// reload between the two would make, and the even rotation of n2, applied to
// each pair in registers (one sweep instead of four; the same arithmetic,
// operator by operator, as separate sweeps or separate launches, so results
// do not depend on where a run is cut into launches).  The mask is one
// factor per r row, so the elements of a row in no even pair (l = 0 when
// the row's pairs start at 1, the last l when the count left is odd) are
// scaled and renormalised on their own.
template <typename R>
__device__ __forceinline__ void rotate_mask_rotate_even(const Tile<R>& tl, int rows, int nl, int j0, int jj, int lane,
                                                        int lanes, const RotTab<R>& tb, R tau1, R ef1, R tau2, R ef2,
                                                        bool do_mask, bool keep) {
    if (jj < rows) {
        const int j = j0 + jj;
        const int l0 = int((int64_t(j) * nl) & 1);
        const R rqj = tb.rq[j];
        const R m = do_mask ? tb.mask[j] : R(1);
        for (int l = l0 + 2 * lane; l + 1 < nl; l += 2 * lanes) {
            const int k0 = l * ROT_ROWS + jj, k1 = (l + 1) * ROT_ROWS + jj;
            const R c = tb.cl[l] * rqj;
            typename Tile<R>::Pair p = tl.load(k0, k1);
            R cm1, s;
            rot_coeffs(tau1 * (c * ef1), cm1, s);
            Tile<R>::rot(p, cm1, s);
            Tile<R>::quant(p);
            if (do_mask) {
                Tile<R>::scale(p, m);
                Tile<R>::quant(p);
            }
            Tile<R>::renorm(p, keep);
            Tile<R>::quant(p);
            rot_coeffs(tau2 * (c * ef2), cm1, s);
            Tile<R>::rot(p, cm1, s);
            tl.put(k0, k1, p);
        }
        if (lane == 0) {
            if (l0 == 1) {
                if (do_mask) tl.scale(jj, m);
                tl.renorm(jj, keep);
            }
            if (((nl - l0) & 1) && nl - 1 >= l0) {
                const int k = (nl - 1) * ROT_ROWS + jj;
                if (do_mask) tl.scale(k, m);
                tl.renorm(k, keep);
            }
        }
    }
    __syncthreads();
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
__device__ void reduce_tile(const ion_sh_sim& S, const Tile<R>& tl, int rows, int nl, int j0, int tile_idx,
                            double* scratch) {
    const int nq = 1 + 2 * S.n_states;
    double acc = 0.0;
    for (int f = threadIdx.x; f < nl * ROT_ROWS; f += blockDim.x) {
        if ((f & (ROT_ROWS - 1)) >= rows) continue;
        const Cx<double> x = tl.value(f);
        acc += x.re * x.re + x.im * x.im;
    }
    const double tot = block_sum(acc, scratch);
    if (threadIdx.x == 0) S.partials[int64_t(tile_idx) * nq] = tot;
    for (int s = 0; s < S.n_states; ++s) {
        const int ls = S.state_l[s];
        double re = 0.0, im = 0.0;
        const int jj = threadIdx.x;
        if (jj < rows && ls < nl) {
            const Cx<double> x = tl.value(ls * ROT_ROWS + jj);
            // conj(state); a real state reads one double (ai = -0.0, the
            // same arithmetic as its complex128 form)
            const int64_t at = int64_t(s) * S.n_r + j0 + jj;
            const double ar = S.state_real ? S.state_g[at] : S.state_g[2 * at];
            const double ai = S.state_real ? -0.0 : -S.state_g[2 * at + 1];
            re = ar * x.re - ai * x.im;
            im = ar * x.im + ai * x.re;
        }
        const double tr = block_sum(re, scratch);
        const double ti = block_sum(im, scratch);
        if (threadIdx.x == 0) {
            S.partials[int64_t(tile_idx) * nq + 1 + 2 * s] = tr;
            S.partials[int64_t(tile_idx) * nq + 2 + 2 * s] = ti;
        }
    }
}

// Neumaier-compensated sum of the per-tile partials into the data slot (at
// data times), then (ADV_STEP) the time index advance; one CTA per simulation
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

// the tile (complex64: hi and the packed lo, 12 bytes an element), the
// block-sum scratch and the simulation's c_l (staged once per tile: every
// pair of every operator reads its c_l, and from shared memory that read is
// a short one; the global loads cost 9 % of the pass)
template <typename R>
__host__ __device__ inline size_t rot_smem_bytes(int max_nl, int rows) {
    return size_t(max_nl) * rows * (sizeof(Cx<R>) + (std::is_same<R, float>::value ? 4 : 0)) + 32 * sizeof(double) +
           size_t(max_nl) * sizeof(R);
}

// c_l of the tile's simulation into shared memory (after the block-sum
// scratch); the caller's barrier publishes it
template <typename R>
__device__ __forceinline__ const R* stage_cl(const RotTab<R>& tb, double* scratch, int nl) {
    R* cl = reinterpret_cast<R*>(scratch + 32);
    for (int l = threadIdx.x; l < nl; l += blockDim.x) cl[l] = tb.cl[l];
    return cl;
}

template <typename R>
__global__ void __maxnreg__(sizeof(R) == 8 ? 64 : 48) sh_rot_kernel(ion_sh_plan plan, int mode, int pf_dist) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int si = plan.rot_items[2 * blockIdx.x];
    const int tile_idx = plan.rot_items[2 * blockIdx.x + 1];
    const ion_sh_sim& S = plan.sims[si];
    if (S.gauge != ION_GAUGE_LENGTH) return;  // sh_rot_vel_kernel
    const int64_t t = S.t;
    const int64_t tf = S.t_final;

    bool post = false, do_mask = false, reduce = false, pre = false;
    int64_t n_post = 0, n_pre = 0;
    if (mode == ROT_PRE_ONLY) {
        if (t >= tf) return;
        pre = true;
        n_pre = t + 1;
    } else if (mode == ROT_STEP || mode == ROT_STEP_PRE) {
        if (t >= tf) return;
        post = true;
        n_post = t + 1;
        do_mask = (sizeof(R) == 8 ? static_cast<const void*>(S.mask) : static_cast<const void*>(S.mask32)) != nullptr;
        reduce = is_data_time(t + 1, tf, S.store_every);
        if (mode == ROT_STEP_PRE && t + 1 < tf) {
            pre = true;
            n_pre = t + 2;
        }
    } else if (mode == ROT_REDUCE_ONLY) {
        reduce = is_data_time(t, tf, S.store_every);
        if (!reduce) return;
    }

    const int nr = S.n_r, nl = S.n_l;
    constexpr int rows_max = ROT_ROWS;
    const int j0 = tile_idx * rows_max;
    const int rows = min(rows_max, nr - j0);
    if (rows <= 0) return;
    const size_t tile_elems = size_t(plan.max_n_l) * rows_max;
    Cx<R>* hi = reinterpret_cast<Cx<R>*>(smem_raw);
    Tile<R> tl;
    tl.hi = hi;
    double* scratch;
    if constexpr (Tile<R>::comp) {
        tl.lo = reinterpret_cast<uint32_t*>(hi + tile_elems);
        scratch = reinterpret_cast<double*>(tl.lo + tile_elems);
    } else {
        scratch = reinterpret_cast<double*>(hi + tile_elems);
    }
    Cx<R>* g = static_cast<Cx<R>*>(S.g);
    // complex64 with a stored residual: the tile's compensation word starts
    // from it and is stored back renormalised instead of folded into g
    uint32_t* glo = Tile<R>::comp ? static_cast<uint32_t*>(S.g_lo) : nullptr;
    // the tile by asynchronous copies: every thread's loads are in flight
    // together without holding registers (register loads left the pass
    // waiting on global memory at a third of the DRAM bandwidth)
    for (int f = threadIdx.x; f < nl * ROT_ROWS; f += blockDim.x) {
        const int l = f >> 5, jj = f & (ROT_ROWS - 1);
        if (jj < rows) {
            const int64_t at = int64_t(l) * nr + j0 + jj;
            if constexpr (sizeof(Cx<R>) == 16)
                cp_async16(hi + f, g + at);
            else
                cp_async8(hi + f, g + at);
            if constexpr (Tile<R>::comp) {
                if (glo)
                    cp_async4(tl.lo + f, glo + at);
                else
                    tl.lo[f] = 0u;
            }
        }
    }
    cp_async_commit();
    if (pf_dist > 0 && blockIdx.x + pf_dist < plan.n_rot_items) prefetch_rot_item<R>(plan, blockIdx.x + pf_dist);
    // the step's scalars (FP64 tables, converted to R) and c_l while the tile lands
    const R tp = post ? R(S.tau[n_post]) : R(0), ep = post ? R(S.efield[n_post]) : R(0);
    const R tq = pre ? R(S.tau[n_pre]) : R(0), eq = pre ? R(S.efield[n_pre]) : R(0);
    RotTab<R> tb = RotTab<R>::make(S);
    tb.cl = stage_cl(tb, scratch, nl);
    cp_async_wait<0>();
    __syncthreads();

    const int jj = threadIdx.x & (ROT_ROWS - 1), lane = threadIdx.x >> 5;
    const int lanes = blockDim.x >> 5;
    if (post && pre && !reduce) {
        // odd(n+1); even(n+1), mask, even(n+2) in one sweep; odd(n+2)
        rotate_rows<R>(tl, rows, nl, j0, jj, lane, lanes, 1, tb, tp, ep);
        rotate_mask_rotate_even<R>(tl, rows, nl, j0, jj, lane, lanes, tb, tp, ep, tq, eq, do_mask, glo != nullptr);
        rotate_rows<R>(tl, rows, nl, j0, jj, lane, lanes, 1, tb, tq, eq);
        post = pre = do_mask = false;
    }
    if (post) {
        rotate_rows<R>(tl, rows, nl, j0, jj, lane, lanes, 1, tb, tp, ep);  // odd
        rotate_rows<R>(tl, rows, nl, j0, jj, lane, lanes, 0, tb, tp, ep);  // even
    }
    if (do_mask) {
        for (int f = threadIdx.x; f < nl * ROT_ROWS; f += blockDim.x) {
            const int jm = f & (ROT_ROWS - 1);
            if (jm < rows) tl.scale(f, tb.mask[j0 + jm]);
        }
        __syncthreads();
    }
    if (reduce) {
        reduce_tile<R>(S, tl, rows, nl, j0, tile_idx, scratch);
        __syncthreads();
    }
    if (post && pre && Tile<R>::comp) {  // as if stored and reloaded between the two (see above)
        for (int f = threadIdx.x; f < nl * ROT_ROWS; f += blockDim.x)
            if ((f & (ROT_ROWS - 1)) < rows) tl.renorm(f, glo != nullptr);
        __syncthreads();
    }
    if (pre) {
        rotate_rows<R>(tl, rows, nl, j0, jj, lane, lanes, 0, tb, tq, eq);  // even
        rotate_rows<R>(tl, rows, nl, j0, jj, lane, lanes, 1, tb, tq, eq);  // odd
    }
    if (mode != ROT_REDUCE_ONLY) {
#pragma unroll 4
        for (int f = threadIdx.x; f < nl * ROT_ROWS; f += blockDim.x) {
            const int l = f >> 5, j2 = f & (ROT_ROWS - 1);
            if (j2 < rows) tl.store(f, g, glo, int64_t(l) * nr + j0 + j2);
        }
    }
}

// ---------------------------------------------------------------------------
// Velocity gauge (ion_sh_sim.gauge == ION_GAUGE_VELOCITY): the same tiles of
// ROT_ROWS r rows x all l, loaded with VEL_HALO rows on each side.  h2 couples
// r and r +- 1, and a tile applies at most 8 such operators per launch (4
// after the solve of step n, 4 before the solve of step n+1), each of which
// leaves one more row at a cut edge wrong; so with 8 halo rows the interior
// rows are exact, and only they are stored and reduced.
// ---------------------------------------------------------------------------
constexpr int VEL_HALO = 8;
constexpr int VEL_ROWS = ROT_ROWS + 2 * VEL_HALO;

// h1 of parity ``parity`` (F-order pairs of l at each r) on every loaded row
template <typename R>
__device__ __forceinline__ void vel_h1(const Tile<R>& tl, int jlo, int jhi, int nl, int r0, int parity,
                                       const RotTab<R>& tb, R tau, R afield) {
    const int span = jhi - jlo;
    const int pairs = nl >> 1;
    for (int idx = threadIdx.x; idx < span * pairs; idx += blockDim.x) {
        const int jj = jlo + idx % span;
        const int j = r0 + jj;  // mesh row
        const int l = int((int64_t(j) * nl + parity) & 1) + 2 * (idx / span);
        if (l + 1 >= nl) continue;
        R cm1, s;
        rot_coeffs(tau * ((tb.cl[l] * R(l + 1)) * (tb.rq[j] * afield)), cm1, s);
        tl.rotate_real(l * VEL_ROWS + jj, (l + 1) * VEL_ROWS + jj, cm1, s);
    }
    __syncthreads();
}

// h2 of l-pair parity lp and r-pair parity rp: per block, the pairs
// ((l, r), (l+1, r+1)) and ((l+1, r), (l, r+1)) turn by [[cos, sin], [-sin, cos]]
template <typename R>
__device__ __forceinline__ void vel_h2(const Tile<R>& tl, int jlo, int jhi, int nl, int r0, int lp, int rp,
                                       const RotTab<R>& tb, const R* h2r, R tau, R afield) {
    const int lpairs = (nl - lp) >> 1;
    const int rpairs = (VEL_ROWS - rp) >> 1;
    for (int idx = threadIdx.x; idx < lpairs * rpairs; idx += blockDim.x) {
        const int jj = rp + 2 * (idx % rpairs);  // r0 is even, so row parity = jj parity
        const int l = lp + 2 * (idx / rpairs);
        if (jj < jlo || jj + 1 >= jhi) continue;
        R cm1, s;
        rot_coeffs(tau * ((tb.cl[l] * h2r[r0 + jj]) * afield), cm1, s);
        tl.rotate_real(l * VEL_ROWS + jj, (l + 1) * VEL_ROWS + jj + 1, cm1, s);
        tl.rotate_real((l + 1) * VEL_ROWS + jj, l * VEL_ROWS + jj + 1, cm1, s);
    }
    __syncthreads();
}

template <typename R> struct VelTab;
template <> struct VelTab<double> {
    __device__ static const double* h2r(const ion_sh_sim& S) { return S.h2r; }
};
template <> struct VelTab<float> {
    __device__ static const float* h2r(const ion_sh_sim& S) { return S.h2r32; }
};

template <typename R>
__global__ void __launch_bounds__(ROT_ROWS * ROT_LANES) sh_rot_vel_kernel(ion_sh_plan plan, int mode) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int si = plan.rot_items[2 * blockIdx.x];
    const int tile_idx = plan.rot_items[2 * blockIdx.x + 1];
    const ion_sh_sim& S = plan.sims[si];
    if (S.gauge != ION_GAUGE_VELOCITY) return;
    const int64_t t = S.t;
    const int64_t tf = S.t_final;
    bool post = false, do_mask = false, reduce = false, pre = false;
    int64_t n_post = 0, n_pre = 0;
    if (mode == ROT_PRE_ONLY) {
        if (t >= tf) return;
        pre = true;
        n_pre = t + 1;
    } else if (mode == ROT_STEP || mode == ROT_STEP_PRE) {
        if (t >= tf) return;
        post = true;
        n_post = t + 1;
        do_mask = (sizeof(R) == 8 ? static_cast<const void*>(S.mask) : static_cast<const void*>(S.mask32)) != nullptr;
        reduce = is_data_time(t + 1, tf, S.store_every);
        if (mode == ROT_STEP_PRE && t + 1 < tf) {
            pre = true;
            n_pre = t + 2;
        }
    } else if (mode == ROT_REDUCE_ONLY) {
        reduce = is_data_time(t, tf, S.store_every);
        if (!reduce) return;
    }
    const int nr = S.n_r, nl = S.n_l;
    const int j0 = tile_idx * ROT_ROWS;
    const int rows = min(ROT_ROWS, nr - j0);
    if (rows <= 0) return;
    const int r0 = j0 - VEL_HALO;  // mesh row of tile row 0
    const int jlo = max(0, -r0), jhi = min(VEL_ROWS, nr - r0);
    const size_t tile_elems = size_t(plan.max_n_l) * VEL_ROWS;
    Cx<R>* hi = reinterpret_cast<Cx<R>*>(smem_raw);
    Tile<R> tl;
    tl.hi = hi;
    double* scratch;
    if constexpr (Tile<R>::comp) {
        tl.lo = reinterpret_cast<uint32_t*>(hi + tile_elems);
        scratch = reinterpret_cast<double*>(tl.lo + tile_elems);
    } else {
        scratch = reinterpret_cast<double*>(hi + tile_elems);
    }
    Cx<R>* g = static_cast<Cx<R>*>(S.g);
    uint32_t* glo = Tile<R>::comp ? static_cast<uint32_t*>(S.g_lo) : nullptr;
    const int span = jhi - jlo;
    for (int f = threadIdx.x; f < nl * span; f += blockDim.x) {  // asynchronous, as in sh_rot_kernel
        const int l = f / span, jj = jlo + f % span;
        const int64_t at = int64_t(l) * nr + r0 + jj;
        if constexpr (sizeof(Cx<R>) == 16)
            cp_async16(hi + l * VEL_ROWS + jj, g + at);
        else
            cp_async8(hi + l * VEL_ROWS + jj, g + at);
        if constexpr (Tile<R>::comp) {
            if (glo)
                cp_async4(tl.lo + l * VEL_ROWS + jj, glo + at);
            else
                tl.lo[l * VEL_ROWS + jj] = 0u;
        }
    }
    cp_async_commit();
    RotTab<R> tb = RotTab<R>::make(S);
    tb.cl = stage_cl(tb, scratch, nl);
    cp_async_wait<0>();
    __syncthreads();
    const R* h2r = VelTab<R>::h2r(S);
    if (post) {  // reversed(S): h2 (odd, odd) ... (even, even), h1 odd, h1 even
        const R tau = R(S.tau[n_post]), af = R(S.efield[n_post]);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 1, 1, tb, h2r, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 1, 0, tb, h2r, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 0, 1, tb, h2r, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 0, 0, tb, h2r, tau, af);
        vel_h1<R>(tl, jlo, jhi, nl, r0, 1, tb, tau, af);
        vel_h1<R>(tl, jlo, jhi, nl, r0, 0, tb, tau, af);
    }
    if (do_mask) {
        for (int f = threadIdx.x; f < nl * span; f += blockDim.x) {
            const int l = f / span, jj = jlo + f % span;
            tl.scale(l * VEL_ROWS + jj, tb.mask[r0 + jj]);
        }
        __syncthreads();
    }
    if (reduce) {  // interior rows
        const int nq = 1 + 2 * S.n_states;
        double acc = 0.0;
        for (int f = threadIdx.x; f < nl * rows; f += blockDim.x) {
            const Cx<double> x = tl.value((f / rows) * VEL_ROWS + VEL_HALO + f % rows);
            acc += x.re * x.re + x.im * x.im;
        }
        const double tot = block_sum(acc, scratch);
        if (threadIdx.x == 0) S.partials[int64_t(tile_idx) * nq] = tot;
        for (int q = 0; q < S.n_states; ++q) {
            const int ls = S.state_l[q];
            double re = 0.0, im = 0.0;
            const int jj = threadIdx.x;
            if (jj < rows && ls < nl) {
                const Cx<double> x = tl.value(ls * VEL_ROWS + VEL_HALO + jj);
                const int64_t at = int64_t(q) * nr + j0 + jj;
                const double ar = S.state_real ? S.state_g[at] : S.state_g[2 * at];
                const double ai = S.state_real ? -0.0 : -S.state_g[2 * at + 1];
                re = ar * x.re - ai * x.im;
                im = ar * x.im + ai * x.re;
            }
            const double tr = block_sum(re, scratch);
            const double ti = block_sum(im, scratch);
            if (threadIdx.x == 0) {
                S.partials[int64_t(tile_idx) * nq + 1 + 2 * q] = tr;
                S.partials[int64_t(tile_idx) * nq + 2 + 2 * q] = ti;
            }
        }
        __syncthreads();
    }
    if (pre) {  // S: h1 even, h1 odd, h2 (even, even) ... (odd, odd)
        const R tau = R(S.tau[n_pre]), af = R(S.efield[n_pre]);
        vel_h1<R>(tl, jlo, jhi, nl, r0, 0, tb, tau, af);
        vel_h1<R>(tl, jlo, jhi, nl, r0, 1, tb, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 0, 0, tb, h2r, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 0, 1, tb, h2r, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 1, 0, tb, h2r, tau, af);
        vel_h2<R>(tl, jlo, jhi, nl, r0, 1, 1, tb, h2r, tau, af);
    }
    if (post || pre || do_mask) {
        for (int f = threadIdx.x; f < nl * rows; f += blockDim.x) {
            const int l = f / rows, jr = f % rows;
            tl.store(l * VEL_ROWS + VEL_HALO + jr, g, glo, int64_t(l) * nr + j0 + jr);
        }
    }
}


// ---------------------------------------------------------------------------
// Coupled lines (kinetic_energy_from_hamiltonian, complex128).  The radial
// operator joins the last r of line l to the first r of line l+1 with H
// coupling p (hcross).  With A = A_bd + i C and B = B_bd + C (C those
// couplings, tau included), the step x = A^-1 (1 - i B) psi is
//     x = u - i A_bd^-1 C (psi + x),   u = A_bd^-1 (1 - i B_bd) psi,
// u being what the per-line solve leaves in g.  C (psi + x) lives on the line
// ends only, so with s_l = A_l^-1 e_first, t_l = A_l^-1 e_last and c = -i tau p
//     x_l = u_l + c (beta_l s_l + alpha_l t_l),
//     beta_l = psi_{l-1,last} + x_{l-1,last},  alpha_l = psi_{l+1,first} + x_{l+1,first},
// and the 2 n_l line-end values (a_l, b_l) = (x_{l,first}, x_{l,last}) solve a
// block-tridiagonal system of 2x2 blocks (block Thomas, one thread).
// ---------------------------------------------------------------------------
__global__ void sh_edge_save_kernel(ion_sh_plan plan) {
    const ion_sh_sim& S = plan.sims[blockIdx.x];
    if (!S.spike_s || !S.edge || S.t >= S.t_final) return;
    const int nr = S.n_r;
    const Cx<double>* g = static_cast<const Cx<double>*>(S.g);
    Cx<double>* e = static_cast<Cx<double>*>(S.edge);
    for (int l = threadIdx.x; l < S.n_l; l += blockDim.x) {
        e[2 * l] = ld(g + int64_t(l) * nr);
        e[2 * l + 1] = ld(g + int64_t(l) * nr + nr - 1);
    }
}

struct Mat2 {
    Cx<double> a, b, c, d;  // [[a, b], [c, d]]
};
__device__ __forceinline__ Mat2 inv2(const Mat2& m) {
    const Cx<double> r = crecip(m.a * m.d - m.b * m.c);
    return Mat2{m.d * r, -(m.b * r), -(m.c * r), m.a * r};
}

// one CTA per simulation, one thread: the line ends (shared memory: n_l x
// (G 2x2, h 2) complex), then c beta_l and c alpha_l into edge[2 n_l ..]
__global__ void sh_coupled_solve_kernel(ion_sh_plan plan) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const ion_sh_sim& S = plan.sims[blockIdx.x];
    if (!S.spike_s || !S.spike_t || !S.edge || S.t >= S.t_final || S.n_l < 2) return;
    const int L = S.n_l, nr = S.n_r;
    Cx<double>* G = reinterpret_cast<Cx<double>*>(smem_raw);  // [L][4]
    Cx<double>* H = G + 4 * L;                                 // [L][2]
    Cx<double>* e = static_cast<Cx<double>*>(S.edge);
    Cx<double>* cf = e + 2 * L;                                 // [L][2]: c beta_l, c alpha_l
    const Cx<double>* g = static_cast<const Cx<double>*>(S.g);
    const Cx<double>* sp = static_cast<const Cx<double>*>(S.spike_s);
    const Cx<double>* tp = static_cast<const Cx<double>*>(S.spike_t);
    const Cx<double> c = {0.0, -S.tau[S.t + 1] * S.hcross};
    const Cx<double> zero = {0.0, 0.0}, one = {1.0, 0.0};
    if (threadIdx.x == 0) {
        // row l: z_l + P_l z_{l-1} + Q_l z_{l+1} = r_l with z = (a, b),
        // P_l = -c [[0, s0], [0, sN]], Q_l = -c [[t0, 0], [tN, 0]]
        Mat2 Gp = {zero, zero, zero, zero};
        Cx<double> hp0 = zero, hp1 = zero;
        for (int l = 0; l < L; ++l) {
            const int64_t f = int64_t(l) * nr, k = f + nr - 1;
            const Cx<double> s0 = ld(sp + f), sN = ld(sp + k), t0 = ld(tp + f), tN = ld(tp + k);
            const Cx<double> pb = l > 0 ? e[2 * (l - 1) + 1] : zero;      // psi_{l-1,last}
            const Cx<double> pa = l + 1 < L ? e[2 * (l + 1)] : zero;      // psi_{l+1,first}
            Cx<double> r0 = ld(g + f) + c * (s0 * pb + t0 * pa);
            Cx<double> r1 = ld(g + k) + c * (sN * pb + tN * pa);
            // D = I - P_l G_{l-1}; r -= P_l h_{l-1}: P_l picks the b row of G and h
            Mat2 D = {one, zero, zero, one};
            if (l > 0) {
                const Cx<double> ps0 = -(c * s0), psN = -(c * sN);
                D.a = D.a - ps0 * Gp.c;
                D.b = D.b - ps0 * Gp.d;
                D.c = D.c - psN * Gp.c;
                D.d = D.d - psN * Gp.d;
                r0 = r0 - ps0 * hp1;
                r1 = r1 - psN * hp1;
            }
            const Mat2 Di = inv2(D);
            // G_l = D^-1 Q_l (Q_l has only a first column), h_l = D^-1 r
            const Cx<double> q0 = l + 1 < L ? -(c * t0) : zero, q1 = l + 1 < L ? -(c * tN) : zero;
            Gp = Mat2{Di.a * q0 + Di.b * q1, zero, Di.c * q0 + Di.d * q1, zero};
            hp0 = Di.a * r0 + Di.b * r1;
            hp1 = Di.c * r0 + Di.d * r1;
            G[4 * l] = Gp.a;
            G[4 * l + 2] = Gp.c;
            H[2 * l] = hp0;
            H[2 * l + 1] = hp1;
        }
        // back substitution: z_l = h_l - G_l z_{l+1} (G_l has only a first column)
        Cx<double> an = zero;  // a_{l+1}
        for (int l = L - 1; l >= 0; --l) {
            const Cx<double> a = H[2 * l] - G[4 * l] * an, b = H[2 * l + 1] - G[4 * l + 2] * an;
            H[2 * l] = a;
            H[2 * l + 1] = b;
            an = a;
        }
        for (int l = 0; l < L; ++l) {
            const Cx<double> beta = l > 0 ? e[2 * (l - 1) + 1] + H[2 * (l - 1) + 1] : zero;
            const Cx<double> alpha = l + 1 < L ? e[2 * (l + 1)] + H[2 * (l + 1)] : zero;
            cf[2 * l] = c * beta;
            cf[2 * l + 1] = c * alpha;
        }
    }
}

// grid (n_sims, chunks): x = u + c beta_l s_l + c alpha_l t_l on every point
__global__ void __launch_bounds__(256) sh_coupled_apply_kernel(ion_sh_plan plan) {
    const ion_sh_sim& S = plan.sims[blockIdx.x];
    if (!S.spike_s || !S.spike_t || !S.edge || S.t >= S.t_final || S.n_l < 2) return;
    const int L = S.n_l, nr = S.n_r;
    Cx<double>* g = static_cast<Cx<double>*>(S.g);
    const Cx<double>* sp = static_cast<const Cx<double>*>(S.spike_s);
    const Cx<double>* tp = static_cast<const Cx<double>*>(S.spike_t);
    const Cx<double>* cf = static_cast<const Cx<double>*>(S.edge) + 2 * L;
    const int64_t n = int64_t(L) * nr;
    for (int64_t k = int64_t(blockIdx.y) * blockDim.x + threadIdx.x; k < n; k += int64_t(gridDim.y) * blockDim.x) {
        const int l = int(k / nr);
        st(g + k, ld(g + k) + cf[2 * l] * ld(sp + k) + cf[2 * l + 1] * ld(tp + k));
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// rows per thread of the radial solve: the compile-time register capacity
// of sh_cn_pipelined; plan.cn_rows = 0 selects the default
template <typename R> struct ShRows;
template <> struct ShRows<double> {
    static bool ok(int r) { return r == 4 || r == 8; }
};
template <> struct ShRows<float> {
    static bool ok(int r) { return r == 4 || r == 8 || r == 16; }
};

// the largest CTA of the radial solve at ``rows`` rows per thread
template <typename R>
static int sh_max_threads(int rows) {
    return rows == 4 ? sh_cn_max_threads<R, 4>() : 512;
}

template <typename R>
static int sh_rows(const ion_sh_plan* p) {
    return p->cn_rows == 0 ? ShCfg<R>::MAXM : p->cn_rows;
}
// rows per thread of bucket b (b < 0: the plan's)
template <typename R>
static int sh_bucket_rows(const ion_sh_plan* p, int b) {
    return (b >= 0 && p->cn_bucket_rows[b] != 0) ? p->cn_bucket_rows[b] : sh_rows<R>(p);
}

template <typename R>
static int sh_validate(const ion_sh_plan* p) {
    if (!p || !p->sims || p->n_sims < 0 || p->n_cn_items < 0 || p->n_rot_items < 0 ||
        p->rot_rows <= 0 || p->rot_rows > 32 || p->max_n_l <= 0 || p->max_n_r < 2 ||
        p->cn_threads <= 0 || p->cn_threads > sh_max_threads<R>(sh_rows<R>(p)) || (p->cn_threads & 31) ||
        (p->cn_rows != 0 && !ShRows<R>::ok(p->cn_rows))) {
        set_error("ion_sh: invalid plan");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (p->n_cn_buckets < 0 || p->n_cn_buckets > 8) {
        set_error("ion_sh: invalid bucket count");
        return ION_ERR_INVALID_ARGUMENT;
    }
    for (int b = 0, prev = 0; b < p->n_cn_buckets; ++b) {
        const int th = p->cn_bucket_threads[b];
        const int br = p->cn_bucket_rows[b];
        if (p->cn_bucket_end[b] < prev || p->cn_bucket_end[b] > p->n_cn_items || th <= 0 ||
            (br != 0 && !ShRows<R>::ok(br)) || th > sh_max_threads<R>(sh_bucket_rows<R>(p, b)) || (th & 31)) {
            set_error("ion_sh: invalid bucket %d", b);
            return ION_ERR_INVALID_ARGUMENT;
        }
        prev = p->cn_bucket_end[b];
    }
    if (p->n_cn_buckets > 0 && p->cn_bucket_end[p->n_cn_buckets - 1] != p->n_cn_items) {
        set_error("ion_sh: buckets do not cover the items");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if ((p->flags & (ION_SH_VELOCITY | ION_SH_ONLY_VELOCITY)) &&
        rot_smem_bytes<R>(p->max_n_l, VEL_ROWS) > 200 * 1024) {
        set_error("ion_sh: l_bound %d too large for the velocity-gauge rotation tile", p->max_n_l);
        return ION_ERR_UNSUPPORTED;
    }
    const int rows = sh_rows<R>(p);
    if (int64_t(p->max_n_r) > int64_t(rows) * sh_max_threads<R>(rows) ||
        sh_line_threads(p->max_n_r, rows) > p->cn_threads) {
        set_error("ion_sh: cn_threads %d / rows %d too small for n_r %d", p->cn_threads, rows, p->max_n_r);
        return ION_ERR_INVALID_ARGUMENT;
    }
    return ION_OK;
}

template <typename R>
static size_t rot_smem(const ion_sh_plan* p) {
    return rot_smem_bytes<R>(p->max_n_l, ROT_ROWS);
}

template <typename R>
static int sh_launch_rot(const ion_sh_plan* p, int mode, cudaStream_t s) {
    if (p->n_rot_items == 0) return ION_OK;
    if (!(p->flags & ION_SH_ONLY_VELOCITY)) {
        const size_t smem = rot_smem<R>(p);
        if (int e = ensure_smem_limit((const void*)sh_rot_kernel<R>, 200 * 1024, "sh_rot_kernel")) return e;
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sh_rot_kernel<R>, ROT_ROWS * ROT_LANES, smem);
        sh_rot_kernel<R><<<p->n_rot_items, ROT_ROWS * ROT_LANES, smem, s>>>(*p, mode, per_sm * num_sms());
        if (int e = check_launch("sh_rot_kernel")) return e;
    }
    if (p->flags & (ION_SH_VELOCITY | ION_SH_ONLY_VELOCITY)) {
        const size_t smem = rot_smem_bytes<R>(p->max_n_l, VEL_ROWS);
        if (int e = ensure_smem_limit((const void*)sh_rot_vel_kernel<R>, 200 * 1024, "sh_rot_vel_kernel")) return e;
        sh_rot_vel_kernel<R><<<p->n_rot_items, ROT_ROWS * ROT_LANES, smem, s>>>(*p, mode);
        if (int e = check_launch("sh_rot_vel_kernel")) return e;
    }
    return ION_OK;
}

// one bucket of the radial solve: items [begin, end) at M rows per thread
template <typename R, int M>
static int sh_launch_cn_bucket(const ion_sh_plan* p, int begin, int end, int threads, cudaStream_t s) {
    const int refine = (p->flags & ION_SH_REFINE) && sizeof(R) == 4 ? 1 : 0;
    auto kern = refine ? sh_cn_pipelined<R, M, true> : sh_cn_pipelined<R, M, false>;
    if (int e = ensure_smem_limit((const void*)kern, 200 * 1024, "sh_cn_pipelined")) return e;
    int dbuf = 1;
    size_t smem = sh_cn_pipelined_smem<R>(threads, M, refine, 1);
    if (smem > 200 * 1024) {
        dbuf = 0;
        smem = sh_cn_pipelined_smem<R>(threads, M, refine, 0);
    }
    if (smem > 200 * 1024) {
        set_error("ion_sh: radial line too long for shared memory");
        return ION_ERR_UNSUPPORTED;
    }
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem);
    const int grid = std::min(end - begin, std::max(per_sm, 1) * num_sms());
    kern<<<grid, threads, smem, s>>>(*p, begin, end, dbuf);
    return check_launch("sh_cn_pipelined");
}

template <typename R>
static int sh_launch_cn_rows(const ion_sh_plan* p, int rows, int begin, int end, int threads, cudaStream_t s);
template <>
int sh_launch_cn_rows<double>(const ion_sh_plan* p, int rows, int begin, int end, int threads, cudaStream_t s) {
    return rows == 4 ? sh_launch_cn_bucket<double, 4>(p, begin, end, threads, s)
                     : sh_launch_cn_bucket<double, 8>(p, begin, end, threads, s);
}
template <>
int sh_launch_cn_rows<float>(const ion_sh_plan* p, int rows, int begin, int end, int threads, cudaStream_t s) {
    switch (rows) {
        case 4: return sh_launch_cn_bucket<float, 4>(p, begin, end, threads, s);
        case 8: return sh_launch_cn_bucket<float, 8>(p, begin, end, threads, s);
        default: return sh_launch_cn_bucket<float, 16>(p, begin, end, threads, s);
    }
}

// every bucket (or all items at cn_threads) with its own rows per thread.
// The buckets hold different lines, so under stream capture they run side by
// side: bucket 0 on the caller's stream, the others on side streams forked
// from it and joined back (graph edges).  CTAs of different buckets then
// share SMs (a CTA of long lines leaves registers that a CTA of short lines
// can use) and one bucket's tail overlaps the next one's work.  Uncaptured
// calls launch the buckets in stream order: there the cross-stream event
// waits of every step cost more than the overlap gains (a served mix of
// batches on several streams took 18.3-18.8 s forked, 15.7-15.8 s in order).
// The side streams are made on an uncaptured call, for use by later captures.
template <typename R>
static int sh_launch_cn(const ion_sh_plan* p, cudaStream_t s) {
    if (p->n_cn_items == 0) return ION_OK;
    const int nb = p->n_cn_buckets;
    ForkJoin* fj = nb > 1 ? fork_join(s) : nullptr;
    if (fj) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
            cudaGetLastError();
            cs = cudaStreamCaptureStatusNone;
        }
        if (cs != cudaStreamCaptureStatusActive) fj = nullptr;
    }
    if (fj && cudaEventRecord(fj->fork, s) != cudaSuccess) return check_launch("sh_launch_cn fork");
    int begin = 0;
    for (int b = 0; b < (nb > 0 ? nb : 1); ++b) {
        const int end = nb > 0 ? p->cn_bucket_end[b] : p->n_cn_items;
        const int threads = nb > 0 ? p->cn_bucket_threads[b] : p->cn_threads;
        const int rows = sh_bucket_rows<R>(p, nb > 0 ? b : -1);
        cudaStream_t sb = (fj && b > 0) ? fj->s[b - 1] : s;
        if (sb != s && cudaStreamWaitEvent(sb, fj->fork, 0) != cudaSuccess) return check_launch("sh_launch_cn fork");
        if (end > begin)
            if (int e = sh_launch_cn_rows<R>(p, rows, begin, end, threads, sb)) return e;
        if (sb != s && cudaEventRecord(fj->join[b - 1], sb) != cudaSuccess) return check_launch("sh_launch_cn join");
        begin = end;
    }
    for (int b = 1; fj && b < nb; ++b)
        if (cudaStreamWaitEvent(s, fj->join[b - 1], 0) != cudaSuccess) return check_launch("sh_launch_cn join");
    return ION_OK;
}

// the radial phase: the line solves, and for plans with coupled lines
// (complex128) the line ends saved before and the coupling applied after
template <typename R>
static int sh_radial_phase(const ion_sh_plan* p, cudaStream_t s) {
    const bool coupled = (p->flags & ION_SH_COUPLED) && sizeof(R) == 8 && p->n_sims > 0;
    if (coupled) {
        sh_edge_save_kernel<<<p->n_sims, 128, 0, s>>>(*p);
        if (int e = check_launch("sh_edge_save_kernel")) return e;
    }
    if (int e = sh_launch_cn<R>(p, s)) return e;
    if (coupled) {
        const size_t smem = size_t(p->max_n_l) * 6 * sizeof(Cx<double>);
        if (smem > 200 * 1024) {
            set_error("ion_sh: l_bound %d too large for the coupled-line fix-up", p->max_n_l);
            return ION_ERR_UNSUPPORTED;
        }
        if (int e = ensure_smem_limit((const void*)sh_coupled_solve_kernel, 200 * 1024, "sh_coupled_solve_kernel"))
            return e;
        sh_coupled_solve_kernel<<<p->n_sims, 32, smem, s>>>(*p);
        if (int e = check_launch("sh_coupled_solve_kernel")) return e;
        sh_coupled_apply_kernel<<<dim3(p->n_sims, 32), 256, 0, s>>>(*p);
        if (int e = check_launch("sh_coupled_apply_kernel")) return e;
    }
    return ION_OK;
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
        if (int e = sh_radial_phase<R>(p, s)) return e;
        if (int e = sh_launch_rot<R>(p, k + 1 < n_steps ? ROT_STEP_PRE : ROT_STEP, s)) return e;
        sh_advance_kernel<<<p->n_sims, 32, 0, s>>>(*p, ADV_STEP);
        if (int e = check_launch("sh_advance_kernel")) return e;
    }
    return ION_OK;
}

// one kernel of the step sequence, for per-kernel timing and custom drivers
template <typename R>
static int sh_phase(const ion_sh_plan* p, int phase, void* stream) {
    if (int e = sh_validate<R>(p)) return e;
    if (p->n_sims == 0) return ION_OK;
    cudaStream_t s = as_stream(stream);
    switch (phase) {
        case ION_SH_PHASE_PRE: return sh_launch_rot<R>(p, ROT_PRE_ONLY, s);
        case ION_SH_PHASE_CN: return sh_radial_phase<R>(p, s);
        case ION_SH_PHASE_ROT: return sh_launch_rot<R>(p, ROT_STEP, s);
        case ION_SH_PHASE_ROT_PRE: return sh_launch_rot<R>(p, ROT_STEP_PRE, s);
        case ION_SH_PHASE_ADVANCE:
            sh_advance_kernel<<<p->n_sims, 32, 0, s>>>(*p, ADV_STEP);
            return check_launch("sh_advance_kernel");
        default:
            set_error("ion_sh: unknown phase %d", phase);
            return ION_ERR_INVALID_ARGUMENT;
    }
}

// The row-sum remainders of the c64x radial step (ion_sh_sim.row_lo): one
// CTA per (simulation, l) line.  The FP32 coefficients are formed exactly as
// the solve forms them (ShCnCoef32 and load_chunk), so the remainder is of
// exactly the values the solve uses; their sum is exact in FP64.
__global__ void __launch_bounds__(256) sh_row_lo_kernel(ion_sh_plan plan) {
    const int si = plan.cn_items[2 * blockIdx.x];
    const int l = plan.cn_items[2 * blockIdx.x + 1];
    const ion_sh_sim& S = plan.sims[si];
    if (!S.row_lo || !S.kinv || !S.cent || !S.hoff || !S.kinv32 || !S.cent32 || !S.hoff32) return;
    const int n = S.n_r;
    const int64_t tn = S.t < S.t_final ? S.t + 1 : S.t_final;
    const double tau = S.tau[tn > 0 ? tn : 1];
    const float tau32 = float(tau);
    const float ll1 = float(l) * float(l + 1);
    const float c032 = l == 0 ? S.corr0_32 : 0.f;
    const double ll1d = double(l) * double(l + 1);
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        float h = fmaf(ll1, S.cent32[i], S.kinv32[i]);
        if (i == 0) h = h + c032;
        const float bd = tau32 * h;
        const float bo = i < n - 1 ? tau32 * S.hoff32[i] : 0.f;
        const float a0 = i > 0 ? tau32 * S.hoff32[i - 1] : 0.f;
        const double sum32 = (double(bd) + double(a0)) + double(bo);
        double row = S.kinv[i] + ll1d * S.cent[i];
        if (i == 0 && l == 0) row += S.corr0;
        if (i > 0) row += S.hoff[i - 1];
        if (i < n - 1) row += S.hoff[i];
        const uint32_t w = lo_pack(Cx<float>{float(tau * row - sum32), 0.f});
        S.row_lo[int64_t(l) * n + i] = uint16_t(w & 0xffffu);
    }
}

static int sh_row_lo(const ion_sh_plan* p, void* stream) {
    if (int e = sh_validate<float>(p)) return e;
    if (p->n_cn_items == 0) return ION_OK;
    sh_row_lo_kernel<<<p->n_cn_items, 256, 0, as_stream(stream)>>>(*p);
    return check_launch("sh_row_lo_kernel");
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
int ion_sh_split_phase_c128(const ion_sh_plan* plan, int phase, void* stream) {
    return sh_phase<double>(plan, phase, stream);
}
int ion_sh_split_phase_c64(const ion_sh_plan* plan, int phase, void* stream) {
    return sh_phase<float>(plan, phase, stream);
}
int ion_sh_reduce_c128(const ion_sh_plan* plan, void* stream) { return sh_reduce<double>(plan, stream); }
int ion_sh_reduce_c64(const ion_sh_plan* plan, void* stream) { return sh_reduce<float>(plan, stream); }
int ion_sh_row_lo_c64(const ion_sh_plan* plan, void* stream) { return sh_row_lo(plan, stream); }
int64_t ion_sh_max_n_r_c128(void) { return int64_t(ShCfg<double>::MAXM) * ShCfg<double>::MAX_T; }
int64_t ion_sh_max_n_r_c64(void) { return int64_t(ShCfg<float>::MAXM) * ShCfg<float>::MAX_T; }

}  // extern "C"
