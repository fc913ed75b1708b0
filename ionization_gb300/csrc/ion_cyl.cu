// Cylindrical slice mesh, length gauge, alternating-direction implicit step:
// CylindricalSliceMesh (ionization/mesh/meshes.py:509-607),
// CylindricalSliceLengthGaugeOperators (ionization/mesh/mesh_operators.py:550-640),
// AlternatingDirectionImplicit (ionization/mesh/evolution_methods.py:46-77).
// The operator sequence per step is [E(H_rho), I(H_z), E(H_z), I(H_rho)]
// (H order rho, z from kinetic_energy, mesh_operators.py:556-559).
//
// psi is (n_z, n_rho), rho contiguous.  Each ADI pass
//     x = (1 + i tau H_line)^-1 (1 - i tau H_other) psi
// is solved in increment form,
//     (1 + i tau H_line) (x - psi) = -i tau (H_line + H_other) psi,
// by the block partition + PCR solver (ion_cn_solver.cuh):
//   cyl_zpass_kernel    one CTA per rho column j: the column is staged in
//                       shared memory, the H_rho stencil reads the two
//                       neighbouring columns from global memory; writes g_tmp;
//   cyl_rhopass_kernel  one CTA per z row i: rows i-1, i, i+1 of g_tmp
//                       staged in shared memory (coalesced); writes g (mask).
#include "ion_common.cuh"
#include "ion_cn_solver.cuh"

namespace ion {

constexpr int CYL_M = 8;
constexpr int CYL_MAX_T = 512;

__host__ __device__ inline int cyl_threads(int n) { return (n + CYL_M - 1) / CYL_M; }

// the optional diagonal terms: hz_d / hr_d and the field term 0.5 E zq
__device__ __forceinline__ double cyl_field(const ion_cyl_mesh* m, int i, int j, double hf) {
    if (m->zq_pt) return hf * m->zq_pt[int64_t(i) * m->n_rho + j];
    return m->zq ? hf * m->zq[i] : 0.0;
}
// the rho off-diagonal multiplier of row i
__device__ __forceinline__ double cyl_rrow(const ion_cyl_mesh* m, int i) {
    return m->hr_off_row ? m->hr_off_row[i] : 1.0;
}
__device__ __forceinline__ double cyl_hz_d(const ion_cyl_mesh* m, int i, int j) {
    return m->hz_d ? m->hz_d[int64_t(i) * m->n_rho + j] : 0.0;
}
// the z off-diagonal multiplier of column j (1, or hz_off_col[j] E)
__device__ __forceinline__ double cyl_zcol(const ion_cyl_mesh* m, int j, double ef) {
    return m->hz_off_col ? m->hz_off_col[j] * ef : 1.0;
}

// The coefficients are formed in FP64 from the FP64 tables and rounded to
// the working type R (complex64: FP32 sweeps, as the spherical-harmonic and
// line complex64 forms).

// z column j: tau H_z and the H_rho stencil from global memory
template <typename R>
struct ZCoef {
    const ion_cyl_mesh* m;
    int j;
    double tau, hf, zc;  // hf = 0.5 * E, zc = cyl_zcol(m, j, E)
    __device__ __forceinline__ void operator()(int i, R& bo, R& bd) const {
        const int nz = m->n_z;
        if (i >= nz) {
            bo = R(0);
            bd = R(0);
            return;
        }
        bd = R(tau * (cyl_hz_d(m, i, j) + cyl_field(m, i, j, hf)));
        bo = (i < nz - 1) ? R(tau * (m->hz_off[i] * zc)) : R(0);
    }
};

template <typename R>
struct ZExtra {
    const ion_cyl_mesh* m;
    const Cx<R>* g;
    const Cx<R>* line;
    int T, j;
    double tau, hf;
    template <typename RR>
    __device__ __forceinline__ Cx<R> get(int i) const {
        const int nz = m->n_z, nr = m->n_rho;
        if (i >= nz) return Cx<R>{R(0), R(0)};
        const Cx<R>* row = g + int64_t(i) * nr;
        const Cx<R> p = line[islot<CYL_M>(i, T)];
        const R hd = R(m->hr_d[int64_t(i) * nr + j] + cyl_field(m, i, j, hf));
        const double rr = cyl_rrow(m, i);
        Cx<R> v = {hd * p.re, hd * p.im};
        if (j > 0) {
            const Cx<R> q = ld(row + j - 1);
            const R o = R(m->hr_off[j - 1] * rr);
            v = Cx<R>{v.re + o * q.re, v.im + o * q.im};
        }
        if (j < nr - 1) {
            const Cx<R> q = ld(row + j + 1);
            const R o = R(m->hr_off[j] * rr);
            v = Cx<R>{v.re + o * q.re, v.im + o * q.im};
        }
        return Cx<R>{R(tau) * v.re, R(tau) * v.im};
    }
};

template <typename R>
struct CylAddOut {
    Cx<R>* line;
    int T;
    __device__ __forceinline__ void operator()(int i, Cx<R> d) const {
        Cx<R>* p = line + islot<CYL_M>(i, T);
        *p = *p + d;
    }
};

template <typename R>
__global__ void __launch_bounds__(512) cyl_zpass_kernel(ion_cyl_mesh mesh, const Cx<R>* g, Cx<R>* gout,
                                                        int64_t tnext, int bthreads, int do_mask) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int j = blockIdx.x;
    const int nz = mesh.n_z, nr = mesh.n_rho;
    const int T = cyl_threads(nz);
    Cx<R>* line = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* red = line + bthreads * CYL_M;
    for (int i = threadIdx.x; i < T * CYL_M; i += blockDim.x)
        line[islot<CYL_M>(i, T)] = (i < nz) ? ld(g + int64_t(i) * nr + j) : Cx<R>{R(0), R(0)};
    __syncthreads();
    const double tau = mesh.tau[tnext], hf = 0.5 * mesh.efield[tnext];
    const double zc = cyl_zcol(&mesh, j, mesh.efield[tnext]);
    block_cn_solve<R, CYL_M>(T, threadIdx.x, R(1), line, red, ZCoef<R>{&mesh, j, tau, hf, zc},
                             ZExtra<R>{&mesh, g, line, T, j, tau, hf}, CylAddOut<R>{line, T});
    __syncthreads();
    for (int i = threadIdx.x; i < nz; i += blockDim.x) {
        Cx<R> x = line[islot<CYL_M>(i, T)];
        if (do_mask && mesh.mask) {
            const R mk = R(mesh.mask[int64_t(i) * nr + j]);
            x = Cx<R>{x.re * mk, x.im * mk};
        }
        st(gout + int64_t(i) * nr + j, x);
    }
}

// rho row i: tau H_rho and the H_z stencil from the staged neighbour rows
template <typename R>
struct RCoef {
    const ion_cyl_mesh* m;
    int i;
    double tau, hf;
    __device__ __forceinline__ void operator()(int j, R& bo, R& bd) const {
        const int nr = m->n_rho;
        if (j >= nr) {
            bo = R(0);
            bd = R(0);
            return;
        }
        bd = R(tau * (m->hr_d[int64_t(i) * nr + j] + cyl_field(m, i, j, hf)));
        bo = (j < nr - 1) ? R(tau * (m->hr_off[j] * cyl_rrow(m, i))) : R(0);
    }
};

template <typename R>
struct RExtra {
    const ion_cyl_mesh* m;
    const Cx<R>* up;    // row i-1 (natural layout)
    const Cx<R>* down;  // row i+1
    const Cx<R>* line;  // row i (interleaved)
    int T, i;
    double tau, hf, ef;
    template <typename RR>
    __device__ __forceinline__ Cx<R> get(int j) const {
        const int nz = m->n_z, nr = m->n_rho;
        if (j >= nr) return Cx<R>{R(0), R(0)};
        const Cx<R> p = line[islot<CYL_M>(j, T)];
        const R hd = R(cyl_hz_d(m, i, j) + cyl_field(m, i, j, hf));
        const double zc = cyl_zcol(m, j, ef);
        Cx<R> v = {hd * p.re, hd * p.im};
        if (i > 0) {
            const R o = R(m->hz_off[i - 1] * zc);
            v = Cx<R>{v.re + o * up[j].re, v.im + o * up[j].im};
        }
        if (i < nz - 1) {
            const R o = R(m->hz_off[i] * zc);
            v = Cx<R>{v.re + o * down[j].re, v.im + o * down[j].im};
        }
        return Cx<R>{R(tau) * v.re, R(tau) * v.im};
    }
};

template <typename R>
__global__ void __launch_bounds__(512) cyl_rhopass_kernel(ion_cyl_mesh mesh, const Cx<R>* gin, Cx<R>* g,
                                                          int64_t tnext, int bthreads, int do_mask) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.x;
    const int nz = mesh.n_z, nr = mesh.n_rho;
    const int T = cyl_threads(nr);
    Cx<R>* up = reinterpret_cast<Cx<R>*>(smem_raw);
    Cx<R>* down = up + nr;
    Cx<R>* line = down + nr;
    Cx<R>* red = line + bthreads * CYL_M;
    const Cx<R> zero = {R(0), R(0)};
    for (int j = threadIdx.x; j < T * CYL_M; j += blockDim.x) {
        if (j < nr) {
            up[j] = (i > 0) ? ld(gin + int64_t(i - 1) * nr + j) : zero;
            down[j] = (i < nz - 1) ? ld(gin + int64_t(i + 1) * nr + j) : zero;
        }
        line[islot<CYL_M>(j, T)] = (j < nr) ? ld(gin + int64_t(i) * nr + j) : zero;
    }
    __syncthreads();
    const double tau = mesh.tau[tnext], hf = 0.5 * mesh.efield[tnext];
    block_cn_solve<R, CYL_M>(T, threadIdx.x, R(1), line, red, RCoef<R>{&mesh, i, tau, hf},
                             RExtra<R>{&mesh, up, down, line, T, i, tau, hf, mesh.efield[tnext]},
                             CylAddOut<R>{line, T});
    __syncthreads();
    for (int j = threadIdx.x; j < nr; j += blockDim.x) {
        Cx<R> x = line[islot<CYL_M>(j, T)];
        if (do_mask && mesh.mask) {
            const R mk = R(mesh.mask[int64_t(i) * nr + j]);
            x = Cx<R>{x.re * mk, x.im * mk};
        }
        st(g + int64_t(i) * nr + j, x);
    }
}

template <typename R>
static size_t zpass_smem(int threads) {
    return size_t(threads) * CYL_M * sizeof(Cx<R>) + pcr_smem_bytes<R>(threads);
}
template <typename R>
static size_t rhopass_smem(int nr, int threads) {
    return 2 * size_t(nr) * sizeof(Cx<R>) + size_t(threads) * CYL_M * sizeof(Cx<R>) + pcr_smem_bytes<R>(threads);
}

template <typename R>
static int cyl_validate(const ion_cyl_mesh* m) {
    if (!m || m->n_z < 2 || m->n_rho < 2 || !m->hz_off || !m->hr_d || !m->hr_off || !m->tau || !m->efield ||
        (m->order != ION_ADI_STRIDED_FIRST && m->order != ION_ADI_CONTIG_FIRST)) {
        set_error("ion_cyl: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int Tz = cyl_threads(m->n_z), Tr = cyl_threads(m->n_rho);
    const int bz = (Tz + 31) / 32 * 32, br = (Tr + 31) / 32 * 32;
    if (bz > CYL_MAX_T || br > CYL_MAX_T || zpass_smem<R>(bz) > 200 * 1024 ||
        rhopass_smem<R>(m->n_rho, br) > 200 * 1024) {
        set_error("ion_cyl: mesh %d x %d too large for one CTA per line", m->n_z, m->n_rho);
        return ION_ERR_UNSUPPORTED;
    }
    if (int e = ensure_smem_limit((const void*)cyl_zpass_kernel<R>, 200 * 1024, "cyl_zpass_kernel")) return e;
    if (int e = ensure_smem_limit((const void*)cyl_rhopass_kernel<R>, 200 * 1024, "cyl_rhopass_kernel")) return e;
    return ION_OK;
}

// one pass: implicit along the strided axis (z) or along the contiguous one (rho)
template <typename R>
static int cyl_pass(const ion_cyl_mesh* m, const Cx<R>* gin, Cx<R>* gout, int64_t tn, int implicit_axis, int do_mask,
                    cudaStream_t s) {
    if (implicit_axis == ION_ADI_PASS_STRIDED) {
        const int bz = (cyl_threads(m->n_z) + 31) / 32 * 32;
        cyl_zpass_kernel<R><<<m->n_rho, bz, zpass_smem<R>(bz), s>>>(*m, gin, gout, tn, bz, do_mask);
        return check_launch("cyl_zpass_kernel");
    }
    const int br = (cyl_threads(m->n_rho) + 31) / 32 * 32;
    cyl_rhopass_kernel<R><<<m->n_z, br, rhopass_smem<R>(m->n_rho, br), s>>>(*m, gin, gout, tn, br, do_mask);
    return check_launch("cyl_rhopass_kernel");
}

template <typename R>
static int cyl_run(const ion_cyl_mesh* m, void* g, void* g_tmp, int64_t t0, int64_t n_steps, void* stream) {
    if (!g || !g_tmp || n_steps < 0 || t0 < 0) {
        set_error("ion_cyl: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (int e = cyl_validate<R>(m)) return e;
    cudaStream_t s = as_stream(stream);
    auto* gg = static_cast<Cx<R>*>(g);
    auto* gt = static_cast<Cx<R>*>(g_tmp);
    // ION_ADI_CONTIG_FIRST: E(H_z) I(H_rho), then E(H_rho) I(H_z) and the mask;
    // ION_ADI_STRIDED_FIRST: E(H_rho) I(H_z), then E(H_z) I(H_rho) and the mask
    const int first = m->order == ION_ADI_CONTIG_FIRST ? ION_ADI_PASS_CONTIG : ION_ADI_PASS_STRIDED;
    const int second = first == ION_ADI_PASS_CONTIG ? ION_ADI_PASS_STRIDED : ION_ADI_PASS_CONTIG;
    for (int64_t k = 0; k < n_steps; ++k) {
        const int64_t tn = t0 + k + 1;
        if (int e = cyl_pass<R>(m, gg, gt, tn, first, 0, s)) return e;
        if (int e = cyl_pass<R>(m, gt, gg, tn, second, 1, s)) return e;
    }
    return ION_OK;
}

template <typename R>
static int cyl_pass_entry(const ion_cyl_mesh* m, const void* g_in, void* g_out, int64_t t_next, int implicit_axis,
                          int apply_mask, void* stream) {
    if (!g_in || !g_out || g_in == g_out || t_next < 1 ||
        (implicit_axis != ION_ADI_PASS_STRIDED && implicit_axis != ION_ADI_PASS_CONTIG)) {
        set_error("ion_cyl_adi_pass: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (int e = cyl_validate<R>(m)) return e;
    return cyl_pass<R>(m, static_cast<const Cx<R>*>(g_in), static_cast<Cx<R>*>(g_out), t_next, implicit_axis,
                       apply_mask ? 1 : 0, as_stream(stream));
}

}  // namespace ion

using namespace ion;

extern "C" {
int ion_cyl_adi_run_c128(const ion_cyl_mesh* mesh, void* g, void* g_tmp, int64_t t0, int64_t n_steps,
                         void* stream) {
    return cyl_run<double>(mesh, g, g_tmp, t0, n_steps, stream);
}
int ion_cyl_adi_run_c64(const ion_cyl_mesh* mesh, void* g, void* g_tmp, int64_t t0, int64_t n_steps, void* stream) {
    return cyl_run<float>(mesh, g, g_tmp, t0, n_steps, stream);
}
int ion_cyl_adi_pass_c128(const ion_cyl_mesh* mesh, const void* g_in, void* g_out, int64_t t_next,
                          int implicit_axis, int apply_mask, void* stream) {
    return cyl_pass_entry<double>(mesh, g_in, g_out, t_next, implicit_axis, apply_mask, stream);
}
int ion_cyl_adi_pass_c64(const ion_cyl_mesh* mesh, const void* g_in, void* g_out, int64_t t_next, int implicit_axis,
                         int apply_mask, void* stream) {
    return cyl_pass_entry<float>(mesh, g_in, g_out, t_next, implicit_axis, apply_mask, stream);
}
int64_t ion_cyl_max_points_c128(void) { return int64_t(CYL_M) * CYL_MAX_T; }
int64_t ion_cyl_max_points_c64(void) { return int64_t(CYL_M) * CYL_MAX_T; }
}
