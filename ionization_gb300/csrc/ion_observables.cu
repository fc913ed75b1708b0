// Position expectation values and partial norms of a mesh wavefunction, for
// the ZExpectationValue, RExpectationValue, NormWithinRadius and
// NormBySphericalHarmonic datastores (ionization/mesh/data.py:344-464).
//
//   ion_weighted_norms_*  out[k] = weight * sum_i w[k][i] |g_i|^2 for a few
//                         FP64 weight vectors (line and cylindrical meshes:
//                         w = z, r, or the indicator r <= R, as
//                         QuantumMesh.expectation_value with an element-wise
//                         operator and NormWithinRadius.store compute them,
//                         meshes.py:206-237, data.py:407-425).
//   ion_sh_observables_*  on the (l, r) spherical-harmonic mesh, in one pass:
//                         <r> = dr sum |g|^2 r_j;
//                         <z> = dr sum 2 Re(conj(g_{l,j}) g_{l+1,j}) c_l r_j, the
//                           F-order off-diagonal z operator of
//                           SphericalHarmonicLengthGaugeOperators.z
//                           (mesh_operators.py:1086-1104);
//                         the norm of each l (SphericalHarmonicMesh.norm_by_l,
//                         meshes.py:1133-1136);
//                         the norm within each radius R_k (rows r_j <= R_k).
//   ion_expectation_*     <g|H|g> for up to four Hermitian operators made of
//                         a diagonal and nearest-neighbour couplings along
//                         the two axes of the mesh, in one pass (the
//                         InternalEnergyExpectationValue and
//                         TotalEnergyExpectationValue datastores,
//                         data.py:290-340, QuantumMesh.expectation_value
//                         with internal_hamiltonian and
//                         interaction_hamiltonian, meshes.py:206-229,
//                         mesh_operators.py:244-298);
//   ion_sh_radial_current_*  the radial probability current through each
//                         shell r_j, split into z > 0 and z < 0 (the
//                         DirectionalRadialProbabilityCurrent datastore,
//                         data.py:467-530, with
//                         SphericalHarmonicMesh.get_radial_probability_
//                         current_density_mesh__spatial, meshes.py:1358-1371).
// The complex64 state may carry its stored residual (g + g_lo).  Stage 1
// writes FP64 partials per CTA (per row tile for the SH form); stage 2 adds
// them in CTA order with Neumaier compensation, so results do not depend on
// scheduling.
#include "ion_common.cuh"

namespace ion {

constexpr int OBS_THREADS = 256;
constexpr int OBS_BLOCKS = 304;
constexpr int OBS_MAX_W = 8;      // weight vectors per call
constexpr int OBS_MAX_RADII = 8;  // radii per SH call
constexpr int OBS_ROWS = 32;      // r rows per SH tile

__device__ __forceinline__ double obs_warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// block sum, valid in thread 0; every thread calls it
__device__ __forceinline__ double obs_block_sum(double v, double* sh) {
    v = obs_warp_sum(v);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < int(blockDim.x >> 5); ++i) r += sh[i];
    return r;
}

// glo: the stored residual of a complex64 state (packed bf16x2), or NULL
template <typename R>
__device__ __forceinline__ Cx<double> value_at(const Cx<R>* g, const uint32_t* glo, int64_t k) {
    const Cx<R> x = ld(g + k);
    Cx<double> v = {double(x.re), double(x.im)};
    if (glo) {
        const Cx<float> e = lo_unpack(glo[k]);
        v.re += double(e.re);
        v.im += double(e.im);
    }
    return v;
}

template <typename R>
__device__ __forceinline__ double abs2_at(const Cx<R>* g, const uint32_t* glo, int64_t k) {
    const Cx<double> v = value_at(g, glo, k);
    return v.re * v.re + v.im * v.im;
}

template <typename R>
__global__ void __launch_bounds__(OBS_THREADS) weighted_stage1(int64_t n, const Cx<R>* g, const uint32_t* glo, int nw,
                                                               const double* w, double* part) {
    __shared__ double sh[32];
    double acc[OBS_MAX_W];
#pragma unroll
    for (int k = 0; k < OBS_MAX_W; ++k) acc[k] = 0.0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
        const double p = abs2_at(g, glo, i);
#pragma unroll
        for (int k = 0; k < OBS_MAX_W; ++k)
            if (k < nw) acc[k] += w[int64_t(k) * n + i] * p;
    }
    for (int k = 0; k < nw; ++k) {
        const double t = obs_block_sum(acc[k], sh);
        if (threadIdx.x == 0) part[int64_t(blockIdx.x) * nw + k] = t;
    }
}

// sum of the per-CTA (or per-tile) partials in CTA order, Neumaier-compensated
__global__ void obs_stage2(int nparts, int nq, const double* part, double weight, double* out) {
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double sum = 0.0, comp = 0.0;
        for (int b = 0; b < nparts; ++b) {
            const double v = part[int64_t(b) * nq + q];
            const double t = sum + v;
            comp += (fabs(sum) >= fabs(v)) ? (sum - t) + v : (v - t) + sum;
            sum = t;
        }
        out[q] = (sum + comp) * weight;
    }
}

// one CTA per tile of OBS_ROWS rows x all l; warp w takes l = w, w + 8, ...
// and lane jj the row j0 + jj, so a warp's loads are one contiguous segment
template <typename R>
__global__ void __launch_bounds__(OBS_THREADS) sh_obs_stage1(const Cx<R>* g, const uint32_t* glo, int nr, int nl,
                                                             const double* r, const double* cl, int nrad,
                                                             const double* radii, double* part) {
    __shared__ double sh[32];
    const int nq = 2 + nl + nrad;
    const int tile = blockIdx.x;
    const int jj = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const int j = tile * OBS_ROWS + jj;
    const bool row_ok = j < nr;
    const double rj = row_ok ? r[j] : 0.0;
    double acc_r = 0.0, acc_z = 0.0, acc_in[OBS_MAX_RADII];
#pragma unroll
    for (int k = 0; k < OBS_MAX_RADII; ++k) acc_in[k] = 0.0;
    for (int l = warp; l < nl; l += nwarp) {
        double p = 0.0;
        if (row_ok) {
            const Cx<double> x = value_at(g, glo, int64_t(l) * nr + j);
            p = x.re * x.re + x.im * x.im;
            acc_r += p * rj;
#pragma unroll
            for (int k = 0; k < OBS_MAX_RADII; ++k)
                if (k < nrad && rj <= radii[k]) acc_in[k] += p;
            if (l + 1 < nl) {
                const Cx<double> y = value_at(g, glo, int64_t(l + 1) * nr + j);
                acc_z += 2.0 * (x.re * y.re + x.im * y.im) * (cl[l] * rj);
            }
        }
        const double pl = obs_warp_sum(p);  // this tile's rows of line l
        if (jj == 0) part[int64_t(tile) * nq + 2 + l] = pl;
    }
    const double tr = obs_block_sum(acc_r, sh);
    const double tz = obs_block_sum(acc_z, sh);
    if (threadIdx.x == 0) {
        part[int64_t(tile) * nq] = tr;
        part[int64_t(tile) * nq + 1] = tz;
    }
    for (int k = 0; k < nrad; ++k) {
        const double t = obs_block_sum(acc_in[k], sh);
        if (threadIdx.x == 0) part[int64_t(tile) * nq + 2 + nl + k] = t;
    }
}

// <g|H_q|g> partials: grid-stride over the points of the (n_a, n_b) mesh;
// point (i, j) adds d |g_ij|^2 and its couplings to (i, j+1) and (i+1, j):
// 2 Re(conj(g) c g') for a real coupling, -2 c Im(conj(g) g') for an
// imaginary one (H_kl = i c, H_lk = -i c).
struct ExpOps {
    ion_hop op[ION_MAX_HOPS];
    int n;
};

__device__ __forceinline__ double coupling_term(double c, Cx<double> x, Cx<double> y, bool imag) {
    const double re = x.re * y.re + x.im * y.im;  // Re(conj(x) y)
    const double im = x.re * y.im - x.im * y.re;  // Im(conj(x) y)
    return imag ? -2.0 * c * im : 2.0 * c * re;
}

template <typename R>
__global__ void __launch_bounds__(OBS_THREADS) expect_stage1(const Cx<R>* g, const uint32_t* glo, int na, int nb,
                                                             ExpOps ops, double* part) {
    __shared__ double sh[32];
    double acc[ION_MAX_HOPS];
#pragma unroll
    for (int q = 0; q < ION_MAX_HOPS; ++q) acc[q] = 0.0;
    const int64_t n = int64_t(na) * nb;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const int64_t i = k / nb;
        const int j = int(k - i * nb);
        const Cx<double> x = value_at(g, glo, k);
        const double p = x.re * x.re + x.im * x.im;
        const bool ha = i + 1 < na;
        const bool hb = j + 1 < nb, wb = !hb && ha;  // wb: the wrap from (i, n_b-1) to (i+1, 0)
        const Cx<double> yb = (hb || wb) ? value_at(g, glo, k + 1) : Cx<double>{0.0, 0.0};
        const Cx<double> ya = ha ? value_at(g, glo, k + nb) : Cx<double>{0.0, 0.0};
#pragma unroll
        for (int q = 0; q < ION_MAX_HOPS; ++q) {
            if (q >= ops.n) break;
            const ion_hop& o = ops.op[q];
            double v = o.diag ? o.diag[k] * p : 0.0;
            if ((hb || (wb && (o.flags & ION_HOP_WRAP_B))) && o.off_b)
                v += coupling_term(o.off_b[k], x, yb, (o.flags & ION_HOP_IMAG_B) != 0);
            if (ha && o.off_a) v += coupling_term(o.off_a[k], x, ya, (o.flags & ION_HOP_IMAG_A) != 0);
            acc[q] += v;
        }
    }
    for (int q = 0; q < ops.n; ++q) {
        const double t = obs_block_sum(acc[q], sh);
        if (threadIdx.x == 0) part[int64_t(blockIdx.x) * ops.n + q] = t;
    }
}

// The radial current through shell j of a spherical-harmonic mesh, z > 0 and
// z < 0: with u_l = g[l][j] and v_l = od[j] g[l][j+1] - od[j-1] g[l][j-1]
// (the reference's r-current operator, mesh_operators.py:1107-1127: real
// antisymmetric couplings od[j] = hbar / (2 m dr^3) / ((j+1)^2 - 1/4)),
//     out[h][j] = r_j^2 Im(sum_{l,l'} conj(u_l) W_h[l][l'] v_l'),
// W_h[l][l'] = 2 pi dtheta sum over the theta_calc points of hemisphere h of
// sin(theta) Y_l(theta) Y_l'(theta): the reference's theta sum of
// Im(conj(psi(r, theta)) (G psi)(r, theta)) sin(theta) dtheta 2 pi with
// psi(r, theta) = sum_l g_l(r) Y_l(theta) (meshes.py:1497-1517), regrouped
// over l pairs (W symmetric: w = W u, then sum conj(w_l') v_l').  One thread
// per shell.
template <typename R>
__global__ void __launch_bounds__(128) sh_current_kernel(const Cx<R>* g, const uint32_t* glo, int nr, int nl,
                                                         const double* od, const double* r, const double* wpos,
                                                         const double* wneg, double* out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nr) return;
    const double odp = j + 1 < nr ? od[j] : 0.0, odm = j > 0 ? od[j - 1] : 0.0;
    double sp = 0.0, sn = 0.0;
    for (int lp = 0; lp < nl; ++lp) {
        Cx<double> wp = {0.0, 0.0}, wn = {0.0, 0.0};
        for (int l = 0; l < nl; ++l) {
            const Cx<double> u = value_at(g, glo, int64_t(l) * nr + j);
            const double a = wpos[int64_t(lp) * nl + l], b = wneg[int64_t(lp) * nl + l];
            wp.re += a * u.re;
            wp.im += a * u.im;
            wn.re += b * u.re;
            wn.im += b * u.im;
        }
        const int64_t base = int64_t(lp) * nr + j;
        Cx<double> v = {0.0, 0.0};
        if (j + 1 < nr) {
            const Cx<double> y = value_at(g, glo, base + 1);
            v.re += odp * y.re;
            v.im += odp * y.im;
        }
        if (j > 0) {
            const Cx<double> y = value_at(g, glo, base - 1);
            v.re -= odm * y.re;
            v.im -= odm * y.im;
        }
        sp += wp.re * v.im - wp.im * v.re;  // Im(conj(w) v)
        sn += wn.re * v.im - wn.im * v.re;
    }
    const double r2 = r[j] * r[j];
    out[j] = r2 * sp;
    out[nr + j] = r2 * sn;
}

static int weighted_blocks(int64_t n) {
    const int64_t b = (n + OBS_THREADS - 1) / OBS_THREADS;
    return int(b < OBS_BLOCKS ? b : OBS_BLOCKS);
}

template <typename R>
static int weighted_impl(int64_t n, const void* g, const void* g_lo, int32_t nw, const double* w, double weight,
                         double* out, void* scratch, int64_t scratch_bytes, void* stream) {
    if (n < 1 || !g || nw < 1 || nw > OBS_MAX_W || !w || !out || !scratch) {
        set_error("ion_weighted_norms: invalid argument (n >= 1, 1 <= n_w <= %d, pointers set)", OBS_MAX_W);
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int blocks = weighted_blocks(n);
    if (scratch_bytes < int64_t(blocks) * nw * int64_t(sizeof(double))) {
        set_error("ion_weighted_norms: scratch too small");
        return ION_ERR_SCRATCH_TOO_SMALL;
    }
    cudaStream_t s = as_stream(stream);
    double* part = static_cast<double*>(scratch);
    weighted_stage1<R><<<blocks, OBS_THREADS, 0, s>>>(n, static_cast<const Cx<R>*>(g),
                                                      static_cast<const uint32_t*>(g_lo), nw, w, part);
    if (int e = check_launch("weighted_stage1")) return e;
    obs_stage2<<<1, 32, 0, s>>>(blocks, nw, part, weight, out);
    return check_launch("obs_stage2");
}

template <typename R>
static int sh_obs_impl(const void* g, const void* g_lo, int32_t nr, int32_t nl, const double* r, const double* cl,
                       int32_t nrad, const double* radii, double weight, double* out, void* scratch,
                       int64_t scratch_bytes, void* stream) {
    if (!g || nr < 1 || nl < 1 || !r || !cl || nrad < 0 || nrad > OBS_MAX_RADII || (nrad > 0 && !radii) || !out ||
        !scratch) {
        set_error("ion_sh_observables: invalid argument (n_r, n_l >= 1, 0 <= n_radii <= %d, pointers set)",
                  OBS_MAX_RADII);
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int tiles = (nr + OBS_ROWS - 1) / OBS_ROWS;
    const int nq = 2 + nl + nrad;
    if (scratch_bytes < int64_t(tiles) * nq * int64_t(sizeof(double))) {
        set_error("ion_sh_observables: scratch too small");
        return ION_ERR_SCRATCH_TOO_SMALL;
    }
    cudaStream_t s = as_stream(stream);
    double* part = static_cast<double*>(scratch);
    sh_obs_stage1<R><<<tiles, OBS_THREADS, 0, s>>>(static_cast<const Cx<R>*>(g), static_cast<const uint32_t*>(g_lo),
                                                   nr, nl, r, cl, nrad, radii, part);
    if (int e = check_launch("sh_obs_stage1")) return e;
    obs_stage2<<<1, 128, 0, s>>>(tiles, nq, part, weight, out);
    return check_launch("obs_stage2");
}

template <typename R>
static int expect_impl(const void* g, const void* g_lo, int32_t na, int32_t nb, int32_t nops, const ion_hop* ops,
                       double weight, double* out, void* scratch, int64_t scratch_bytes, void* stream) {
    if (!g || na < 1 || nb < 1 || nops < 1 || nops > ION_MAX_HOPS || !ops || !out || !scratch) {
        set_error("ion_expectation: invalid argument (n_a, n_b >= 1, 1 <= n_ops <= %d, pointers set)", ION_MAX_HOPS);
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int64_t n = int64_t(na) * nb;
    const int blocks = weighted_blocks(n);
    if (scratch_bytes < int64_t(blocks) * nops * int64_t(sizeof(double))) {
        set_error("ion_expectation: scratch too small");
        return ION_ERR_SCRATCH_TOO_SMALL;
    }
    ExpOps eo{};
    eo.n = nops;
    for (int q = 0; q < nops; ++q) eo.op[q] = ops[q];
    cudaStream_t s = as_stream(stream);
    double* part = static_cast<double*>(scratch);
    expect_stage1<R><<<blocks, OBS_THREADS, 0, s>>>(static_cast<const Cx<R>*>(g), static_cast<const uint32_t*>(g_lo),
                                                    na, nb, eo, part);
    if (int e = check_launch("expect_stage1")) return e;
    obs_stage2<<<1, 32, 0, s>>>(blocks, nops, part, weight, out);
    return check_launch("obs_stage2");
}

template <typename R>
static int sh_current_impl(const void* g, const void* g_lo, int32_t nr, int32_t nl, const double* od, const double* r,
                           const double* wpos, const double* wneg, double* out, void* stream) {
    if (!g || nr < 1 || nl < 1 || !od || !r || !wpos || !wneg || !out) {
        set_error("ion_sh_radial_current: invalid argument (n_r, n_l >= 1, pointers set)");
        return ION_ERR_INVALID_ARGUMENT;
    }
    sh_current_kernel<R><<<(nr + 127) / 128, 128, 0, as_stream(stream)>>>(
        static_cast<const Cx<R>*>(g), static_cast<const uint32_t*>(g_lo), nr, nl, od, r, wpos, wneg, out);
    return check_launch("sh_current_kernel");
}

}  // namespace ion

using namespace ion;

extern "C" {
int64_t ion_weighted_norms_scratch_bytes(int64_t n, int32_t n_w) {
    return n < 1 || n_w < 1 ? 0 : int64_t(weighted_blocks(n)) * n_w * int64_t(sizeof(double));
}
int ion_weighted_norms_c128(int64_t n, const void* g, int32_t n_w, const double* w, double weight, double* out,
                            void* scratch, int64_t scratch_bytes, void* stream) {
    return weighted_impl<double>(n, g, nullptr, n_w, w, weight, out, scratch, scratch_bytes, stream);
}
int ion_weighted_norms_c64(int64_t n, const void* g, const void* g_lo, int32_t n_w, const double* w, double weight,
                           double* out, void* scratch, int64_t scratch_bytes, void* stream) {
    return weighted_impl<float>(n, g, g_lo, n_w, w, weight, out, scratch, scratch_bytes, stream);
}
int64_t ion_sh_observables_scratch_bytes(int32_t n_r, int32_t n_l, int32_t n_radii) {
    if (n_r < 1 || n_l < 1 || n_radii < 0) return 0;
    return int64_t((n_r + OBS_ROWS - 1) / OBS_ROWS) * (2 + n_l + n_radii) * int64_t(sizeof(double));
}
int ion_sh_observables_c128(const void* g, int32_t n_r, int32_t n_l, const double* r, const double* cl,
                            int32_t n_radii, const double* radii, double weight, double* out, void* scratch,
                            int64_t scratch_bytes, void* stream) {
    return sh_obs_impl<double>(g, nullptr, n_r, n_l, r, cl, n_radii, radii, weight, out, scratch, scratch_bytes,
                               stream);
}
int ion_sh_observables_c64(const void* g, const void* g_lo, int32_t n_r, int32_t n_l, const double* r,
                           const double* cl, int32_t n_radii, const double* radii, double weight, double* out,
                           void* scratch, int64_t scratch_bytes, void* stream) {
    return sh_obs_impl<float>(g, g_lo, n_r, n_l, r, cl, n_radii, radii, weight, out, scratch, scratch_bytes, stream);
}
int64_t ion_expectation_scratch_bytes(int32_t n_a, int32_t n_b, int32_t n_ops) {
    if (n_a < 1 || n_b < 1 || n_ops < 1) return 0;
    return int64_t(weighted_blocks(int64_t(n_a) * n_b)) * n_ops * int64_t(sizeof(double));
}
int ion_expectation_c128(const void* g, int32_t n_a, int32_t n_b, int32_t n_ops, const ion_hop* ops, double weight,
                         double* out, void* scratch, int64_t scratch_bytes, void* stream) {
    return expect_impl<double>(g, nullptr, n_a, n_b, n_ops, ops, weight, out, scratch, scratch_bytes, stream);
}
int ion_expectation_c64(const void* g, const void* g_lo, int32_t n_a, int32_t n_b, int32_t n_ops, const ion_hop* ops,
                        double weight, double* out, void* scratch, int64_t scratch_bytes, void* stream) {
    return expect_impl<float>(g, g_lo, n_a, n_b, n_ops, ops, weight, out, scratch, scratch_bytes, stream);
}
int ion_sh_radial_current_c128(const void* g, int32_t n_r, int32_t n_l, const double* od, const double* r,
                               const double* w_pos, const double* w_neg, double* out, void* stream) {
    return sh_current_impl<double>(g, nullptr, n_r, n_l, od, r, w_pos, w_neg, out, stream);
}
int ion_sh_radial_current_c64(const void* g, const void* g_lo, int32_t n_r, int32_t n_l, const double* od,
                              const double* r, const double* w_pos, const double* w_neg, double* out, void* stream) {
    return sh_current_impl<float>(g, g_lo, n_r, n_l, od, r, w_pos, w_neg, out, stream);
}
}
