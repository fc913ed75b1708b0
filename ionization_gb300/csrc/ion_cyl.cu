// Cylindrical slice mesh, length gauge, alternating-direction implicit step:
// CylindricalSliceMesh (ionization/mesh/meshes.py:509-607),
// CylindricalSliceLengthGaugeOperators (ionization/mesh/mesh_operators.py:550-640),
// AlternatingDirectionImplicit (ionization/mesh/evolution_methods.py:46-77).
// The operator sequence per step is [E(H_rho), I(H_z), E(H_z), I(H_rho)]
// (H order rho, z from kinetic_energy, mesh_operators.py:556-559).
//
// psi is (n_z, n_rho), rho contiguous.  Two passes per step:
//   cyl_zpass_kernel    one CTA per rho column j: rhs = (1 - i tau H_rho) g at
//                       (i, j) read from global memory (three neighbours along
//                       rho), solve along z in shared memory, write g_tmp;
//   cyl_rhopass_kernel  one CTA per z row i: rows i-1, i, i+1 of g_tmp staged
//                       in shared memory (coalesced), rhs = (1 - i tau H_z)
//                       g_tmp, solve along rho, mask, write g.
#include "ion_common.cuh"
#include "ion_solver.cuh"

namespace ion {

constexpr int CYL_MAXM = 8;
constexpr int CYL_MAX_T = 512;

__host__ __device__ inline int cyl_threads(int n) {
    int T = (n + CYL_MAXM - 1) / CYL_MAXM;
    if (T > n / 2) T = n / 2;
    if (T < 1) T = 1;
    return T;
}

struct CylStep {
    double tau, hfield;  // hfield = 0.5 * E (per-direction share of the interaction)
};

// z-line of column j: coefficients of (1 + i tau H_z)
struct ZCoef {
    const ion_cyl_mesh* m;
    int j;
    double tau, ef;
    __device__ void operator()(int64_t i, Cx<double>& a, Cx<double>& b, Cx<double>& c) const {
        const Cx<double> zero = {0.0, 0.0};
        const int nz = m->n_z, nr = m->n_rho;
        a = (i > 0) ? Cx<double>{0.0, tau * m->hz_off[i - 1]} : zero;
        const double hd = m->hz_d[int64_t(i) * nr + j] + 0.5 * (m->zq[i] * ef);
        b = Cx<double>{1.0, tau * hd};
        c = (i < nz - 1) ? Cx<double>{0.0, tau * m->hz_off[i]} : zero;
    }
};

// rhs of the z pass: ((1 - i tau H_rho) g)(i, j), neighbours along rho
struct ZRhs {
    const ion_cyl_mesh* m;
    const Cx<double>* g;
    int j;
    double tau, ef;
    __device__ Cx<double> operator()(int64_t i) const {
        const int nr = m->n_rho;
        const Cx<double>* row = g + int64_t(i) * nr;
        Cx<double> y = {0.0, 0.0};
        if (j > 0) y = mul_ih(-tau * m->hr_off[j - 1], ld(row + j - 1));
        const Cx<double> p = ld(row + j);
        const double hd = -tau * (m->hr_d[int64_t(i) * nr + j] + 0.5 * (m->zq[i] * ef));
        y = y + Cx<double>{p.re - hd * p.im, p.im + hd * p.re};
        if (j < nr - 1) y = y + mul_ih(-tau * m->hr_off[j], ld(row + j + 1));
        return y;
    }
};

struct SmemLineOut {
    Cx<double>* line;
    __device__ void operator()(int64_t i, Cx<double> x) const { line[i] = x; }
};

__global__ void __launch_bounds__(512) cyl_zpass_kernel(ion_cyl_mesh mesh, const Cx<double>* g,
                                                        Cx<double>* gout, int64_t tnext, int T) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int j = blockIdx.x;
    const int nz = mesh.n_z, nr = mesh.n_rho;
    Cx<double>* line = reinterpret_cast<Cx<double>*>(smem_raw);
    Cx<double>* red = line + (nz + 1) / 2 * 2;
    const double tau = mesh.tau[tnext], ef = mesh.efield[tnext];
    block_line_solve<double, CYL_MAXM>(nz, T, threadIdx.x, int(threadIdx.x) < T, red,
                                        ZCoef{&mesh, j, tau, ef}, ZRhs{&mesh, g, j, tau, ef},
                                        SmemLineOut{line});
    __syncthreads();
    for (int i = threadIdx.x; i < nz; i += blockDim.x) st(gout + int64_t(i) * nr + j, line[i]);
}

// rho-line of row i: coefficients of (1 + i tau H_rho)
struct RCoef {
    const ion_cyl_mesh* m;
    int i;
    double tau, ef;
    __device__ void operator()(int64_t j, Cx<double>& a, Cx<double>& b, Cx<double>& c) const {
        const Cx<double> zero = {0.0, 0.0};
        const int nr = m->n_rho;
        a = (j > 0) ? Cx<double>{0.0, tau * m->hr_off[j - 1]} : zero;
        const double hd = m->hr_d[int64_t(i) * nr + j] + 0.5 * (m->zq[i] * ef);
        b = Cx<double>{1.0, tau * hd};
        c = (j < nr - 1) ? Cx<double>{0.0, tau * m->hr_off[j]} : zero;
    }
};

// rhs of the rho pass: ((1 - i tau H_z) g_tmp)(i, j), rows staged in smem
struct RRhs {
    const ion_cyl_mesh* m;
    const Cx<double>* rows;  // [3][n_rho]: rows i-1, i, i+1
    int i;
    double tau, ef;
    __device__ Cx<double> operator()(int64_t j) const {
        const int nz = m->n_z, nr = m->n_rho;
        Cx<double> y = {0.0, 0.0};
        if (i > 0) y = mul_ih(-tau * m->hz_off[i - 1], rows[j]);
        const Cx<double> p = rows[nr + j];
        const double hd = -tau * (m->hz_d[int64_t(i) * nr + j] + 0.5 * (m->zq[i] * ef));
        y = y + Cx<double>{p.re - hd * p.im, p.im + hd * p.re};
        if (i < nz - 1) y = y + mul_ih(-tau * m->hz_off[i], rows[2 * nr + j]);
        return y;
    }
};

__global__ void __launch_bounds__(512) cyl_rhopass_kernel(ion_cyl_mesh mesh, const Cx<double>* gin,
                                                          Cx<double>* g, int64_t tnext, int T) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int i = blockIdx.x;
    const int nz = mesh.n_z, nr = mesh.n_rho;
    Cx<double>* rows = reinterpret_cast<Cx<double>*>(smem_raw);  // 3 * nr
    Cx<double>* line = rows + 3 * nr;                             // nr (output)
    Cx<double>* red = line + (nr + 1) / 2 * 2;
    for (int f = threadIdx.x; f < 3 * nr; f += blockDim.x) {
        const int r = f / nr, j = f - r * nr;
        const int ii = i - 1 + r;
        rows[f] = (ii >= 0 && ii < nz) ? ld(gin + int64_t(ii) * nr + j) : Cx<double>{0.0, 0.0};
    }
    __syncthreads();
    const double tau = mesh.tau[tnext], ef = mesh.efield[tnext];
    block_line_solve<double, CYL_MAXM>(nr, T, threadIdx.x, int(threadIdx.x) < T, red,
                                        RCoef{&mesh, i, tau, ef}, RRhs{&mesh, rows, i, tau, ef},
                                        SmemLineOut{line});
    __syncthreads();
    for (int j = threadIdx.x; j < nr; j += blockDim.x) {
        Cx<double> x = line[j];
        if (mesh.mask) {
            const double mk = mesh.mask[int64_t(i) * nr + j];
            x = Cx<double>{x.re * mk, x.im * mk};
        }
        st(g + int64_t(i) * nr + j, x);
    }
}

static size_t zpass_smem(int nz, int T) { return (size_t(nz) + 1) / 2 * 2 * 16 + pcr_smem_bytes<double>(T); }
static size_t rhopass_smem(int nr, int T) {
    return (3 * size_t(nr) + (size_t(nr) + 1) / 2 * 2) * 16 + pcr_smem_bytes<double>(T);
}

static int cyl_run(const ion_cyl_mesh* m, void* g, void* g_tmp, int64_t t0, int64_t n_steps, void* stream) {
    if (!m || !g || !g_tmp || m->n_z < 2 || m->n_rho < 2 || n_steps < 0 || t0 < 0 || !m->hz_d ||
        !m->hz_off || !m->hr_d || !m->hr_off || !m->zq || !m->tau || !m->efield) {
        set_error("ion_cyl: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int Tz = cyl_threads(m->n_z), Tr = cyl_threads(m->n_rho);
    if (Tz > CYL_MAX_T || Tr > CYL_MAX_T || zpass_smem(m->n_z, Tz) > 200 * 1024 ||
        rhopass_smem(m->n_rho, Tr) > 200 * 1024 ||
        int64_t(m->n_z) > int64_t(CYL_MAXM) * CYL_MAX_T || int64_t(m->n_rho) > int64_t(CYL_MAXM) * CYL_MAX_T) {
        set_error("ion_cyl: mesh %d x %d too large for one CTA per line", m->n_z, m->n_rho);
        return ION_ERR_UNSUPPORTED;
    }
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(cyl_zpass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(cyl_rhopass_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr = true;
    }
    cudaStream_t s = as_stream(stream);
    auto* gg = static_cast<Cx<double>*>(g);
    auto* gt = static_cast<Cx<double>*>(g_tmp);
    const int bz = (Tz + 31) / 32 * 32, br = (Tr + 31) / 32 * 32;
    for (int64_t k = 0; k < n_steps; ++k) {
        const int64_t tn = t0 + k + 1;
        cyl_zpass_kernel<<<m->n_rho, bz, zpass_smem(m->n_z, Tz), s>>>(*m, gg, gt, tn, Tz);
        if (int e = check_launch("cyl_zpass_kernel")) return e;
        cyl_rhopass_kernel<<<m->n_z, br, rhopass_smem(m->n_rho, Tr), s>>>(*m, gt, gg, tn, Tr);
        if (int e = check_launch("cyl_rhopass_kernel")) return e;
    }
    return ION_OK;
}

}  // namespace ion

using namespace ion;

extern "C" {
int ion_cyl_adi_run_c128(const ion_cyl_mesh* mesh, void* g, void* g_tmp, int64_t t0, int64_t n_steps,
                         void* stream) {
    return cyl_run(mesh, g, g_tmp, t0, n_steps, stream);
}
int64_t ion_cyl_max_points_c128(void) { return int64_t(CYL_MAXM) * CYL_MAX_T; }
}
