/*
 * ionization_gb300 — C ABI of the GB300 (sm_103a) mesh time-evolution library.
 *
 * Conventions for every entry point:
 *   - all array arguments are DEVICE pointers owned by the caller; the library
 *     never allocates device memory on these paths (scratch, where needed, is
 *     passed in and its size is given by the matching *_scratch_bytes query);
 *   - complex arrays are interleaved (re, im) pairs: c128 = two doubles,
 *     c64 = two floats;
 *   - ``stream`` is a cudaStream_t (NULL = legacy default stream); work is
 *     enqueued asynchronously and the call returns without synchronising;
 *   - the return value is ION_OK (0) or a negative ION_ERR_* code; a text
 *     description of the last error on the calling thread is available from
 *     ion_last_error().  No C++ exception crosses this boundary;
 *   - calls on distinct streams are independent; a call is thread-safe with
 *     respect to other calls that touch different buffers.
 *
 * Reference interfaces replaced (paths relative to the ionization project):
 *   ion_tdma_*            ionization/cy.pyx:9 ``tdma(matrix, d)`` as called by
 *                         TDMAOperator._apply, ionization/mesh/mesh_operators.py:109-111
 *   ion_line_*_run_*      one LineMesh step, QuantumMesh.evolve
 *                         (ionization/mesh/meshes.py:251-257) with
 *                         AlternatingDirectionImplicit / SplitInteractionOperator
 *                         (ionization/mesh/evolution_methods.py:46-123) over
 *                         LineLengthGaugeOperators (mesh_operators.py:304-341)
 *   ion_sh_split_run_*    one SphericalHarmonicMesh step with
 *                         SplitInteractionOperator (evolution_methods.py:80-123) over
 *                         SphericalHarmonicLengthGaugeOperators (mesh_operators.py:815-1080)
 *   ion_cyl_adi_run_*     one CylindricalSliceMesh ADI step
 *                         (evolution_methods.py:46-77, mesh_operators.py:550-640)
 *   ion_reduce_*          QuantumMesh.inner_product / norm (meshes.py:195-217) and the
 *                         SphericalHarmonicMesh inner-product shortcut (meshes.py:1099-1131)
 *   ion_weighted_norms_*, ion_sh_observables_*
 *                         QuantumMesh.z/r_expectation_value (meshes.py:231-237),
 *                         SphericalHarmonicMesh.norm_by_l (meshes.py:1133-1136),
 *                         NormWithinRadius (data.py:407-425)
 */
#ifndef IONIZATION_GB300_H
#define IONIZATION_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    ION_OK = 0,
    ION_ERR_INVALID_ARGUMENT = -1,
    ION_ERR_CUDA = -2,
    ION_ERR_UNSUPPORTED = -3,
    ION_ERR_SCRATCH_TOO_SMALL = -4,
    ION_ERR_NONFINITE = -5
};

/* Text of the last error raised on the calling thread ("" if none). */
const char *ion_last_error(void);
/* Library ABI version (major * 10000 + minor * 100 + patch). */
int ion_version(void);

/* ------------------------------------------------------------------------
 * Thomas / tridiagonal solves — replaces ionization/cy.pyx:9 tdma(matrix, d)
 *
 * The matrix is given exactly as cy.tdma reads a scipy dia_matrix with offsets
 * (-1, 0, 1) (cy.pyx:18-21):
 *   sub[k]  = A[k+1, k]   k = 0..n-2   (matrix.data[0][:-1])
 *   diag[k] = A[k, k]     k = 0..n-1   (matrix.data[1])
 *   sup[k]  = A[k, k+1]   k = 0..n-2   (matrix.data[2][1:])
 * and x = A^-1 d.  Like cy.tdma there is no pivoting: a zero pivot gives
 * inf/nan in x.  ``x`` may not alias the inputs.
 * ------------------------------------------------------------------------ */

/* Scratch (device bytes) needed by ion_tdma_* for one system of n rows. */
int64_t ion_tdma_scratch_bytes_c128(int64_t n);
int64_t ion_tdma_scratch_bytes_c64(int64_t n);

/* One system of n rows (any n >= 1). */
int ion_tdma_c128(int64_t n, const void *sub, const void *diag, const void *sup, const void *d,
                  void *x, void *scratch, int64_t scratch_bytes, void *stream);
int ion_tdma_c64(int64_t n, const void *sub, const void *diag, const void *sup, const void *d,
                 void *x, void *scratch, int64_t scratch_bytes, void *stream);

/* One system of n rows, like ion_tdma_c128, but taking no scratch argument and
 * allocating nothing.  This entry point has no counterpart in the reference.
 * It is for callers that cannot call cudaMalloc around the solve, for example
 * a host code that runs under a fixed device-memory budget handed out once at
 * start-up, or a time-stepping loop that must not pay the implicit device
 * synchronisation an allocation can cause.  The partition scratch lives in a
 * file-scope device array of 5 MiB (5242880 bytes), enough for
 * n <= ion_tdma_noalloc_max_n_c128() = 65536; larger n is rejected with
 * ION_ERR_INVALID_ARGUMENT.  Every GPU that loads this library holds that
 * array until the process exits.  The first call in each CUDA context (on each
 * device, and again after cudaDeviceReset replaces a device's context) looks
 * up the array's device address (cudaGetSymbolAddress) whatever n is, and
 * caches it with the context's id; make that first call before any stream
 * capture (under capture it returns ION_ERR_INVALID_ARGUMENT instead of doing
 * the lookup).  All calls share the one array: calls whose
 * work overlaps on the GPU (two streams, or two host threads) race on it and
 * must be serialised by the caller.  The array keeps whatever the last call
 * left in it; nothing in it has to start at zero, because each call writes
 * every scratch word before reading it. */
int ion_tdma_noalloc_c128(int64_t n, const void *sub, const void *diag, const void *sup, const void *d,
                          void *x, void *stream);
int64_t ion_tdma_noalloc_max_n_c128(void);

/* nsys independent systems of n rows each, flattened back to back as the mesh
 * operators hand them to cy.tdma (system s = rows [s*n, (s+1)*n) of one long
 * vector of nsys*n rows; sub/sup hold nsys*n-1 entries).  The entries that
 * couple consecutive systems (sub[s*n-1], sup[s*n-1]) must be zero, as the
 * reference operators build them, and are not read.  Requires n >= 2 and
 * n <= ion_tdma_batched_max_n_*(). */
int ion_tdma_batched_c128(int64_t nsys, int64_t n, const void *sub, const void *diag,
                          const void *sup, const void *d, void *x, void *stream);
int ion_tdma_batched_c64(int64_t nsys, int64_t n, const void *sub, const void *diag,
                         const void *sup, const void *d, void *x, void *stream);
int64_t ion_tdma_batched_max_n_c128(void);
int64_t ion_tdma_batched_max_n_c64(void);

/* ------------------------------------------------------------------------
 * Spherical-harmonic mesh, length gauge, split-interaction operator.
 *
 * One step from time index t to t+1 is, as in SplitInteractionOperator
 * (evolution_methods.py:89-123) and QuantumMesh.evolve (meshes.py:251-257):
 *   R_even(t+1), R_odd(t+1), (1 - i tau H0), (1 + i tau H0)^-1,
 *   R_odd(t+1), R_even(t+1), g *= mask(r)
 * with tau = (times[t+1] - times[t]) / 2 and the rotations built from
 * E(times[t+1] + time_step/2) (mesh_operators.py:1011-1013, 1037-1080).  The
 * pairing of the rotations is over the F-order (r-major, l fastest) index of
 * the (l, r) mesh, exactly as the reference builds its even/odd matrices.
 * Between two solves with no data stored in between, R_even(t+1), the mask
 * and R_even(t+2) are applied to each pair in registers in one sweep, with
 * the same arithmetic as separate sweeps, and a complex64 state's (hi, lo)
 * pair is renormalised there as a store and reload between two calls would:
 * results do not depend on how the steps are split into calls, bit for bit.
 *
 * psi of every simulation is stored (n_l, n_r) in C order (r contiguous),
 * the layout of the reference's ``mesh.g``, at its own device pointer.  A batch
 * is any number of simulations of different sizes, each with its own time
 * index ``t`` (kept and advanced on the device), its own final index and its
 * own field table.  Data (norm and test-state inner products, the Norm and
 * InnerProducts datastores, data.py:189-260) are reduced on the device in
 * FP64 at the reference's data times (sims.py:84-90) into ``out_norm`` /
 * ``out_ip`` slots.
 * ------------------------------------------------------------------------ */
typedef struct ion_sh_sim {
    void *g;             /* device psi (n_l, n_r), C order, complex128 or complex64 */
    int32_t n_r, n_l;
    int64_t t;           /* current time index; advanced on the device */
    int64_t t_final;     /* last time index (number of steps of the run) */
    int64_t store_every; /* data at t = 0, t = t_final and t % store_every == 0 if >= 1 */
    /* FP64 tables (complex128 path; the _c64 entry points read hoff, tau and
     * efield of these, and the mask flag from mask32) */
    const double *hd;     /* [n_l*n_r] diagonal of the internal Hamiltonian (C order) */
    const double *hoff;   /* [n_r-1]   its off-diagonal (identical for every l) */
    const double *rq;     /* [n_r]     (-test_charge) * r_j */
    const double *cl;     /* [n_l]     c_l = (l+1)/sqrt((2l+1)(2l+3)) */
    const double *mask;   /* [n_r]     mask(r_j), or NULL for no mask */
    const double *tau;    /* [t_final+1] tau at each time index (entry 0 unused) */
    const double *efield; /* [t_final+1] E(times[t] + time_step/2) (entry 0 unused) */
    /* FP32 tables (complex64 path), rounded from FP64 */
    const float *kinv32;  /* [n_r] -2 p beta(j) + V(r_j)  (diagonal without the l term) */
    const float *cent32;  /* [n_r] hbar^2 / (2 mu r_j^2) */
    const float *hoff32;  /* [n_r-1] */
    const float *rq32;    /* [n_r] */
    const float *cl32;    /* [n_l] */
    const float *mask32;  /* [n_r] or NULL */
    float corr0_32;       /* extra diagonal term at (l=0, j=0) (hydrogen correction) */
    /* data */
    int32_t n_states;
    const int32_t *state_l; /* [n_states] angular momentum of each test state */
    const double *state_g;  /* [n_states*n_r*2] radial g of each test state (complex128) */
    double weight;          /* inner-product multiplier (delta r) */
    double *out_norm;       /* [n_data] */
    double *out_ip;         /* [n_data*n_states*2] complex128 */
    double *partials;       /* [n_tiles * (1 + 2*n_states)] device scratch for reductions */
    int32_t n_tiles;        /* number of row tiles of this simulation */
    int32_t gauge;          /* ION_GAUGE_LENGTH (0) or ION_GAUGE_VELOCITY, see below */
    /* _c64 entry points only, or NULL: the rounding residual of psi, (n_l, n_r)
     * like g, one 32-bit word a point holding its real and imaginary parts as
     * bf16 (real in the low 16 bits, each rounded to nearest even): the
     * ION_LO_BF16X2 format.  psi = g + g_lo carries about 33 significant bits
     * in 12 bytes a point: the arithmetic stays FP32, each step's increment
     * is added to (g, g_lo) with an exact two-sum and the pair is
     * renormalised (|g_lo| <= ulp(g) / 2) when stored, so storing psi no
     * longer rounds it to FP32 precision; the explicit half of the radial
     * step is then formed from neighbour differences and an exact row sum of
     * the same FP32 coefficients, which removes the cancellation of the
     * kinetic terms and keeps the step unitary. */
    void *g_lo;
    /* ION_GAUGE_VELOCITY (SphericalHarmonicVelocityGaugeOperators,
     * mesh_operators.py:1130-1408): the split operators are h1, rotations of
     * F-order l-neighbours at one r by tau A hbar (q/m) c_l (l+1) / r_j, and h2,
     * rotations of the (l, r)-(l+1, r+1) and (l, r+1)-(l+1, r) pairs of each
     * l-pair x r-pair block by tau A c_l h2r[j]; per step h1 even, h1 odd,
     * h2 (even, even), (even, odd), (odd, even), (odd, odd) (l-pair, r-pair
     * parities), the radial solve, the same in reverse.  In this gauge rq
     * (rq32) holds hbar (q/m) / r_j, efield the vector potential A(times[t]),
     * cl the plain c_l. */
    const double *h2r;      /* [n_r-1] hbar (q/m) / (2 dr) alpha(j), or NULL */
    const float *h2r32;
    /* _c64 entry points with g_lo and ION_SH_REFINE only, or NULL: [n_l*n_r]
     * bf16 (C order like g), the row-sum remainder of the radial step per
     * point: tau * (H_ii + H_i,i-1 + H_i,i+1) with the FP64 tables and tau,
     * minus the same sum of the FP32 coefficients the solve forms
     * (tau32 * fma(l(l+1), cent32, kinv32) (+ corr0 at the first point),
     * tau32 * hoff32).  The refinement adds it to the explicit half's exact
     * row sum, so the refined solve converges to the FP64 system instead of
     * to the one the FP32 tables round it to.  That rounding acts as a random
     * potential of ~1e-7 of the kinetic diagonal; in strongly driven runs it
     * moves the final populations by up to ~5e-6.  Filled on the device by
     * ion_sh_row_lo_c64. */
    uint16_t *row_lo;
    /* FP64 per-r tables of the radial diagonal, kinv + l(l+1) cent (+ corr0 at
     * the first point of l = 0): what ion_sh_row_lo_c64 forms row_lo from
     * (NULL when row_lo is) */
    const double *kinv;
    const double *cent;
    double corr0;
    /* _c128 with ION_SH_COUPLED only, or NULL: the radial Hamiltonian of
     * kinetic_energy_from_hamiltonian (mesh_operators.py:863-887) is one
     * tridiagonal over the flattened (l, r) mesh, so it also couples the last
     * r of each l with the first r of the next (hcross).  Each line is solved
     * as before; a fix-up then adds that coupling through the line's spikes
     * spike_s = A_l^-1 e_first and spike_t = A_l^-1 e_last (complex128
     * [n_l*n_r], A_l = 1 + i tau H_l at the uniform time step), solving the
     * 2 n_l line-end values together.  edge: complex128 [4*n_l] scratch
     * (psi's line ends from before the solve, then the coupling
     * coefficients). */
    const void *spike_s;
    const void *spike_t;
    void *edge;
    double hcross;
    /* 1: state_g holds each test state's real radial g, [n_states*n_r]
     * doubles (hydrogen and numeric eigenstates are real); 0: complex128
     * pairs as described above */
    int32_t state_real;
    int32_t pad3_;
} ion_sh_sim;

enum { ION_GAUGE_LENGTH = 0, ION_GAUGE_VELOCITY = 1 };

/* ion_sh_plan.flags: with it, the radial solve of every simulation that carries a
 * stored residual is followed by one step of iterative refinement.  The matrix
 * 1 + i tau H0 is the same at every step, so the FP32 rounding of its
 * elimination is too; unrefined, that fixed error makes the step slightly
 * non-unitary and the norm drifts by ~2e-10 per step.  The refinement solves for
 * the correction with the residual formed from the first solution (about twice
 * the radial-solve time). */
enum { ION_SH_REFINE = 1 };
/* ion_sh_plan.flags: some simulations are in the velocity gauge (their
 * rotation pass runs in its own kernel), or all of them are. */
enum { ION_SH_VELOCITY = 2, ION_SH_ONLY_VELOCITY = 4 };
/* ion_sh_plan.flags: some simulations carry spikes (ion_sh_sim.spike_s): the
 * radial phase saves their line ends before the solve and applies the
 * line-to-line coupling after it (complex128). */
enum { ION_SH_COUPLED = 8 };

typedef struct ion_sh_plan {
    ion_sh_sim *sims;         /* device array [n_sims] */
    int32_t n_sims;
    int32_t max_n_l;          /* largest n_l of the batch */
    int32_t max_n_r;          /* largest n_r of the batch */
    int32_t flags;            /* ION_SH_REFINE: refine the radial solves of the simulations
                                 that carry a stored residual (g_lo) */
    const int32_t *cn_items;  /* device [n_cn_items*2]: (sim, l) handled by one CTA */
    int32_t n_cn_items;
    int32_t cn_threads;       /* CTA size of the radial solve (multiple of 32) */
    const int32_t *rot_items; /* device [n_rot_items*2]: (sim, row tile) */
    int32_t n_rot_items;
    int32_t rot_rows;         /* rows (r points) per tile, <= 64 */
    int32_t cn_rows;          /* rows per thread of the radial solve: 0 = default,
                                 complex128 4 or 8, complex64 4, 8 or 16 */
    int32_t n_cn_buckets;     /* 0: one launch of cn_threads for all items; else the
                                 items are sorted so that bucket b is the range
                                 [cn_bucket_end[b-1], cn_bucket_end[b]) launched with
                                 cn_bucket_threads[b] threads per CTA */
    int32_t cn_bucket_end[8];
    int32_t cn_bucket_threads[8];
    int32_t cn_bucket_rows[8]; /* rows per thread of bucket b's radial solve (its own
                                  CTA shape: cn_bucket_threads[b] * rows >= the bucket's
                                  n_r), or 0 for cn_rows */
} ion_sh_plan;

/* Advance every simulation of the plan by n_steps (fewer for simulations that
 * reach t_final).  Data reductions happen at data times on the way.  With
 * n_cn_buckets > 1 and `stream` under capture, the buckets' radial solves
 * run side by side on side streams forked from `stream` and joined back to
 * it (graph edges); uncaptured calls run them in stream order.  The library
 * makes those side streams once per caller stream, on an uncaptured call: to
 * get the overlap in a captured graph, make one uncaptured call on the
 * capture stream first (else the buckets run in stream order, with the same
 * results). */
int ion_sh_split_run_c128(const ion_sh_plan *plan, int64_t n_steps, void *stream);
int ion_sh_split_run_c64(const ion_sh_plan *plan, int64_t n_steps, void *stream);
/* One kernel of the step sequence (for per-kernel timing or custom drivers):
 * a run of n steps is PRE, then n times (CN, ROT_PRE or ROT on the last, ADVANCE). */
enum {
    ION_SH_PHASE_PRE = 1,     /* rotations before the first radial solve */
    ION_SH_PHASE_CN = 2,      /* radial Crank-Nicolson solve of every (simulation, l) line */
    ION_SH_PHASE_ROT = 3,     /* rotations after the solve, mask, data reductions */
    ION_SH_PHASE_ROT_PRE = 4, /* as ROT, then the rotations before the next solve */
    ION_SH_PHASE_ADVANCE = 5  /* finish reductions, advance every time index */
};
int ion_sh_split_phase_c128(const ion_sh_plan *plan, int phase, void *stream);
int ion_sh_split_phase_c64(const ion_sh_plan *plan, int phase, void *stream);
/* Reduce the data of the current time index (used for t = 0 before the run). */
int ion_sh_reduce_c128(const ion_sh_plan *plan, void *stream);
int ion_sh_reduce_c64(const ion_sh_plan *plan, void *stream);

/* Fill row_lo of every simulation of the plan that carries one (c64x set-up,
 * once per simulation before its first step): per point, tau * (the FP64
 * row sum kinv + l(l+1) cent [+ corr0] + hoff[i-1] + hoff[i]) minus the sum
 * of the FP32 coefficients the radial solve forms for that row, with the
 * solve's own FP32 arithmetic, rounded to bf16; tau = tau[t+1] at the
 * simulation's current time index t (the time step is uniform). */
int ion_sh_row_lo_c64(const ion_sh_plan *plan, void *stream);
/* Largest n_r the radial solve supports in one CTA. */
int64_t ion_sh_max_n_r_c128(void);
int64_t ion_sh_max_n_r_c64(void);

/* ------------------------------------------------------------------------
 * Line mesh, length gauge (LineLengthGaugeOperators, mesh_operators.py:304-341).
 *
 * method ION_LINE_ADI — AlternatingDirectionImplicit (evolution_methods.py:46-77):
 *     (1 + i tau H)^-1 (1 - i tau H),  H = H0 + diag(zq * E(times[t+1]))
 * method ION_LINE_SPLIT — SplitInteractionOperator (evolution_methods.py:80-123):
 *     S (1 + i tau H0)^-1 (1 - i tau H0) S,  S = diag(exp(-i tau zq E(times[t+1])))
 * method ION_LINE_FFT — Fourier split-step, no counterpart in the reference:
 *     P F^-1 K F P,  P = diag(exp(-i tau (vstat + zq E(times[t+1])))),
 *     K = diag(exp(-i 2 tau kin)), F the discrete Fourier transform;
 *     periodic in z, n a power of two.
 * followed by g *= mask (meshes.py:256-257).  One CTA advances one
 * simulation; data reductions are fused into the same pass.  Simulations of
 * different methods may share one plan.
 * ------------------------------------------------------------------------ */
enum { ION_LINE_ADI = 0, ION_LINE_SPLIT = 1, ION_LINE_FFT = 2 };

typedef struct ion_line_sim {
    void *g;          /* device psi [n], complex128 or complex64 */
    int32_t n;
    int32_t method;   /* ION_LINE_ADI or ION_LINE_SPLIT */
    int64_t t, t_final, store_every;
    const double *hd;     /* [n]   diagonal of H0 = kinetic + V */
    const double *hoff;   /* [n-1] off-diagonal of H0 */
    const double *zq;     /* [n]   interaction per unit field, (-z) * test_charge */
    const double *mask;   /* [n] or NULL */
    const double *tau;    /* [t_final+1] */
    const double *efield; /* [t_final+1] E(times[t]) */
    const float *hd32;
    const float *hoff32;
    const float *zq32;
    const float *mask32;
    int32_t n_states;
    int32_t gauge;         /* ION_GAUGE_LENGTH, or ION_GAUGE_VELOCITY (ION_LINE_SPLIT, one CTA, see vcoef) */
    const double *state_g; /* [n_states*n*2] complex128 test states */
    double weight;         /* delta z */
    double *out_norm;      /* [n_data] */
    double *out_ip;        /* [n_data*n_states*2] */
    /* ION_LINE_FFT only (NULL otherwise) */
    const double *vstat;   /* [n] static potential V(z) */
    const double *kin;     /* [n] kinetic energy hbar^2 k^2 / (2 m) of the Fourier mode that the
                              forward transform leaves at position i (bit-reversed order) */
    const void *twiddle;   /* [n] exp(-2 pi i m / n), complex128 for _c128, complex64 for _c64 */
    const float *vstat32;
    /* _c64 entry points with ION_LINE_RESIDUAL: the rounding residual of psi
     * ([n] words in the ION_LO_BF16X2 format of ion_sh_sim.g_lo,
     * psi = g + g_lo), or NULL */
    void *g_lo;
    /* ION_GAUGE_VELOCITY (LineVelocityGaugeOperators, mesh_operators.py:352-427):
     * the split operators are rotations [[cos, sin], [-sin, cos]] of the pairs
     * (2k, 2k+1) (even) and (2k+1, 2k+2) (odd) by tau A vcoef, A = efield[t]
     * the vector potential; per step even, odd, the Crank-Nicolson pair, odd,
     * even.  vcoef = hbar (q/m) / (2 dz).  Runs in one CTA (cluster and
     * residual plans leave such a line untouched). */
    double vcoef;
    /* ION_LINE_RESIDUAL only, or NULL: the low parts of the FP32 tables,
     * x_lo = float(x - double(x32)).  The residual form's explicit half adds
     * them (and the low parts of tau and of the field term) to the FP32 row
     * sums, so its refinement solves the FP64 system. */
    const float *hd_lo32;   /* [n] */
    const float *hoff_lo32; /* [n-1] */
} ion_line_sim;

typedef struct ion_line_plan {
    ion_line_sim *sims; /* device array [n_sims] */
    int32_t n_sims;
    int32_t max_n;
    int32_t threads; /* CTA size (multiple of 32) */
    int32_t cluster; /* CTAs per simulation.  0 or 1: one CTA, n <= ion_line_max_n_*().
                        2..8: a thread-block cluster, the line split into equal
                        segments, n <= cluster * ion_line_max_n_*(); Crank-Nicolson
                        methods only (ION_LINE_FFT simulations are left untouched) */
    int32_t flags;   /* ION_LINE_RESIDUAL (_c64 only): every simulation carries g_lo and
                        is advanced in the residual form: 8 rows per thread,
                        n <= cluster * ion_line_max_n_c64x(), Crank-Nicolson methods,
                        the explicit half in exact-row-sum difference form, one step of
                        iterative refinement of each solve */
    int32_t pad2_;
} ion_line_plan;

/* ION_LINE_HAS_FFT: the plan holds ION_LINE_FFT simulations; their CTAs take
 * the shared memory that caches a step's phase factors (a Fourier line in a
 * plan without the flag is left untouched). */
enum { ION_LINE_RESIDUAL = 1, ION_LINE_HAS_FFT = 2 };

int ion_line_run_c128(const ion_line_plan *plan, int64_t n_steps, void *stream);
int ion_line_run_c64(const ion_line_plan *plan, int64_t n_steps, void *stream);
int ion_line_reduce_c128(const ion_line_plan *plan, void *stream);
int ion_line_reduce_c64(const ion_line_plan *plan, void *stream);
/* Longest line one CTA holds (a cluster of C CTAs holds C times as much);
 * _c64x: in the residual form (ION_LINE_RESIDUAL). */
int64_t ion_line_max_n_c128(void);
int64_t ion_line_max_n_c64(void);
int64_t ion_line_max_n_c64x(void);

/* ------------------------------------------------------------------------
 * Cylindrical slice mesh, length gauge, ADI (CylindricalSliceLengthGaugeOperators,
 * mesh_operators.py:550-640; AlternatingDirectionImplicit, evolution_methods.py:46-77).
 * psi is (n_z, n_rho) in C order (rho contiguous), as the reference's g.
 * One step from t to t+1 with E = E(times[t+1]):
 *   pass 1:  g_tmp = (1 + i tau H_z)^-1 (1 - i tau H_rho) g
 *   pass 2:  g     = (1 + i tau H_rho)^-1 (1 - i tau H_z) g_tmp   (then *= mask)
 * H_d = H0_d + 0.5 zq E on the diagonal (mesh_operators.py:271-298).
 * ------------------------------------------------------------------------ */
typedef struct ion_cyl_mesh {
    int32_t n_z, n_rho;
    const double *hz_d;   /* [n_z*n_rho] diagonal of the internal H_z */
    const double *hz_off; /* [n_z-1] */
    const double *hr_d;   /* [n_z*n_rho] diagonal of the internal H_rho */
    const double *hr_off; /* [n_rho-1] */
    const double *zq;     /* [n_z] */
    const double *mask;   /* [n_z*n_rho] or NULL */
    const double *tau;    /* indexed by time index */
    const double *efield; /* E(times[t]) indexed by time index */
    /* [n_rho] or NULL.  When set, the off-diagonal of H_z between rows i and
     * i+1 in column j is hz_off[i] * hz_off_col[j] * E(t): the interaction of
     * the spherical-harmonic mesh under ADI (mesh_operators.py:1020-1035 with
     * :988-1005), run on this kernel pair with z = l (hz_off = c_l,
     * hz_off_col = -q r_j, hz_d and zq NULL) and rho = r (hr_d, hr_off = the
     * radial H0). */
    const double *hz_off_col;
    /* ION_ADI_STRIDED_FIRST (0): per step E(H_rho), I(H_z), E(H_z), I(H_rho)
     * (the cylinder, whose kinetic operators come rho first); ION_ADI_CONTIG_FIRST:
     * E(H_z), I(H_rho), E(H_rho), I(H_z) (the rectangle mesh, z first,
     * mesh_operators.py:436-437).  The mask follows the step's last pass. */
    int32_t order;
    int32_t pad_;
    /* [n_z] or NULL: the rho off-diagonal of row i is hr_off[j] * hr_off_row[i]
     * (the spherical slice's theta operator, whose coupling scales as
     * 1/(j_r + 1/2)^2 along r) */
    const double *hr_off_row;
    /* [n_z*n_rho] or NULL: when set, the field term of point (i, j) is
     * 0.5 E zq_pt[i*n_rho + j] instead of 0.5 E zq[i] (z varies along both axes) */
    const double *zq_pt;
} ion_cyl_mesh;

enum { ION_ADI_STRIDED_FIRST = 0, ION_ADI_CONTIG_FIRST = 1 };

/* Advance psi from time index t0 by n_steps.  g_tmp is a psi-sized buffer.
 * hz_d and zq may be NULL (no such term).  _c64: psi complex64, the sweeps in
 * FP32 with coefficients rounded from the FP64 tables (the same tables). */
int ion_cyl_adi_run_c128(const ion_cyl_mesh *mesh, void *g, void *g_tmp, int64_t t0,
                         int64_t n_steps, void *stream);
int ion_cyl_adi_run_c64(const ion_cyl_mesh *mesh, void *g, void *g_tmp, int64_t t0,
                        int64_t n_steps, void *stream);

/* One of the two passes of a step, for callers that interleave their own work
 * between them (and for timing each pass): g_out = (1 + i tau H_a)^-1
 * (1 - i tau H_b) g_in with a the implicit axis (ION_ADI_PASS_STRIDED: z, whose
 * lines are strided in memory; ION_ADI_PASS_CONTIG: rho), b the other, tau and
 * E at time index t_next, then g_out *= mask if apply_mask.  ion_cyl_adi_run
 * is the pair in the mesh's order with the mask after the second.  g_in and
 * g_out must not overlap. */
enum { ION_ADI_PASS_STRIDED = 0, ION_ADI_PASS_CONTIG = 1 };
int ion_cyl_adi_pass_c128(const ion_cyl_mesh *mesh, const void *g_in, void *g_out, int64_t t_next,
                          int implicit_axis, int apply_mask, void *stream);
int ion_cyl_adi_pass_c64(const ion_cyl_mesh *mesh, const void *g_in, void *g_out, int64_t t_next,
                         int implicit_axis, int apply_mask, void *stream);
/* Longest line (either axis) of the two passes. */
int64_t ion_cyl_max_points_c128(void);
int64_t ion_cyl_max_points_c64(void);

/* ------------------------------------------------------------------------
 * Eigenpairs of batched real symmetric tridiagonal matrices: the numeric
 * eigenstate basis (SphericalHarmonicMesh.get_numeric_eigenstate_basis,
 * meshes.py:1281-1356, and LineMesh._get_numeric_eigenstate_basis,
 * meshes.py:343-387, which call scipy's eigsh on each single-l Hamiltonian).
 * n_mat matrices of order n >= 2: diag [n_mat*n], off [n_mat*(n-1)], device.
 *   ion_tridiag_count_below: counts[m] = number of eigenvalues of matrix m
 *     below x[m] (Sturm sequence);
 *   ion_tridiag_eigvals: vals[r] = the req_idx[r]-th smallest eigenvalue
 *     (0-based) of matrix req_mat[r], by bisection to the last bits of FP64;
 *   ion_tridiag_eigvecs: vecs[r*n ...] = the eigenvector of matrix req_mat[r]
 *     for eigenvalue vals[r], by inverse iteration (partial pivoting, two
 *     solves from a fixed start), unit 2-norm, sign such that its first
 *     component above 1e-3 of the largest is positive; scratch holds
 *     ion_tridiag_eig_scratch_doubles(n, n_req) doubles.
 * ------------------------------------------------------------------------ */
int64_t ion_tridiag_eig_scratch_doubles(int32_t n, int32_t n_req);
int ion_tridiag_count_below(int32_t n_mat, int32_t n, const double *diag, const double *off, const double *x,
                            int32_t *counts, void *stream);
int ion_tridiag_eigvals(int32_t n_mat, int32_t n, const double *diag, const double *off, int32_t n_req,
                        const int32_t *req_mat, const int32_t *req_idx, double *vals, void *stream);
int ion_tridiag_eigvecs(int32_t n_mat, int32_t n, const double *diag, const double *off, int32_t n_req,
                        const int32_t *req_mat, const double *vals, double *vecs, double *scratch, void *stream);

/* ------------------------------------------------------------------------
 * Norm and inner products on a whole mesh (QuantumMesh.norm / inner_product,
 * meshes.py:195-217):  norm = weight * sum |g|^2,
 * ip[s] = weight * sum conj(states[s]) g, in FP64 with a compensated
 * two-level sum.  ``partials`` is device scratch of
 * ion_reduce_scratch_bytes(M, n_states) bytes.
 * ------------------------------------------------------------------------ */
int64_t ion_reduce_scratch_bytes(int64_t M, int32_t n_states);
int ion_reduce_c128(int64_t M, const void *g, int32_t n_states, const void *states, double weight,
                    double *out_norm, double *out_ip, void *partials, void *stream);
int ion_reduce_c64(int64_t M, const void *g, int32_t n_states, const void *states, double weight,
                   double *out_norm, double *out_ip, void *partials, void *stream);

/* psi of a complex64 state read back as complex128 (the g property of a
 * complex64 mesh, QuantumMesh.g): out[i] = hi[i] + lo[i] in FP64, lo (the
 * stored residual, ION_LO_BF16X2 words) may be NULL.  n complex elements,
 * device pointers. */
int ion_psi_to_c128(int64_t n, const void *hi, const void *lo, void *out, void *stream);
/* The inverse, for uploads: a complex128 psi split into the complex64 hi
 * (rounded to nearest) and, when lo is not NULL, the packed residual
 * (ION_LO_BF16X2) of psi - hi.  n complex elements, device pointers; in may
 * not alias hi or lo. */
int ion_psi_split_c128(int64_t n, const void *in, void *hi, void *lo, void *stream);
/* Many uploaded rows in one launch (a batch's initial states, row by row
 * into each simulation's psi): rows is a DEVICE array of n_rows entries.
 * With hi_c128 = 0 each row is split as by ion_psi_split_c128 (complex64 hi,
 * lo as there, may be NULL); with hi_c128 != 0 it is copied into a
 * complex128 hi and lo is ignored.  Rows may not overlap one another's
 * outputs nor alias their own input; a row with n <= 0 or a NULL in or hi
 * is skipped. */
typedef struct ion_psi_row {
    const void *in;  /* n complex128 */
    void *hi;        /* n complex64 (split) or complex128 (copy) */
    void *lo;        /* n ION_LO_BF16X2 words, or NULL */
    int64_t n;
} ion_psi_row;
int ion_psi_split_rows_c128(int64_t n_rows, const ion_psi_row *rows, int32_t hi_c128, void *stream);

/* ------------------------------------------------------------------------
 * Position expectation values and partial norms (the ZExpectationValue,
 * RExpectationValue, NormWithinRadius and NormBySphericalHarmonic datastores,
 * ionization/mesh/data.py:344-464).  FP64 two-stage sums with a compensated
 * second stage; the complex64 forms accept the stored residual g_lo
 * (ION_LO_BF16X2 words, or NULL).
 *
 * ion_weighted_norms_*: out[k] = weight * sum_i w[k * n + i] |g_i|^2 for
 *   1 <= n_w <= 8 weight vectors (element-wise operators on line and
 *   cylindrical meshes: w = z, r or the indicator r <= R; QuantumMesh.
 *   expectation_value, meshes.py:206-237).
 * ion_sh_observables_*: on the (n_l, n_r) spherical-harmonic mesh,
 *   out[0] = <r>, out[1] = <z> (the F-order off-diagonal z operator of
 *   SphericalHarmonicLengthGaugeOperators.z, mesh_operators.py:1086-1104,
 *   with c_l = cl[l] and r_j = r[j]), out[2 + l] = norm of line l
 *   (SphericalHarmonicMesh.norm_by_l, meshes.py:1133-1136) and
 *   out[2 + n_l + k] = norm of the rows r_j <= radii[k], 0 <= n_radii <= 8;
 *   every entry times ``weight`` (dr).
 * ``scratch`` holds the matching *_scratch_bytes query.
 * ------------------------------------------------------------------------ */
int64_t ion_weighted_norms_scratch_bytes(int64_t n, int32_t n_w);
int ion_weighted_norms_c128(int64_t n, const void *g, int32_t n_w, const double *w, double weight, double *out,
                            void *scratch, int64_t scratch_bytes, void *stream);
int ion_weighted_norms_c64(int64_t n, const void *g, const void *g_lo, int32_t n_w, const double *w,
                           double weight, double *out, void *scratch, int64_t scratch_bytes, void *stream);
int64_t ion_sh_observables_scratch_bytes(int32_t n_r, int32_t n_l, int32_t n_radii);
int ion_sh_observables_c128(const void *g, int32_t n_r, int32_t n_l, const double *r, const double *cl,
                            int32_t n_radii, const double *radii, double weight, double *out, void *scratch,
                            int64_t scratch_bytes, void *stream);
int ion_sh_observables_c64(const void *g, const void *g_lo, int32_t n_r, int32_t n_l, const double *r,
                           const double *cl, int32_t n_radii, const double *radii, double weight, double *out,
                           void *scratch, int64_t scratch_bytes, void *stream);

/* ------------------------------------------------------------------------
 * Energy expectation values (the InternalEnergyExpectationValue and
 * TotalEnergyExpectationValue datastores, data.py:290-340;
 * QuantumMesh.expectation_value, meshes.py:206-229).  A Hermitian operator on
 * an (n_a, n_b) mesh in C order (b contiguous) made of a diagonal and
 * couplings between nearest neighbours along each axis; every table is FP64
 * [n_a*n_b] indexed by the point (i, j) it starts from, or NULL (no such
 * term).  A real coupling c puts c at (k, k') and (k', k); with
 * ION_HOP_IMAG_B / ION_HOP_IMAG_A it is imaginary: i c at (k, k'), -i c at
 * (k', k), k' the neighbour at j+1 or i+1 (LineVelocityGaugeOperators'
 * interaction, mesh_operators.py:358-369).  With ION_HOP_WRAP_B the b
 * coupling of (i, n_b-1) joins it to (i+1, 0): one coupling chain over the
 * flattened mesh (kinetic_energy_from_hamiltonian, mesh_operators.py:863-887).
 *
 * ion_expectation_*: out[q] = weight * <g|H_q|g> for 1 <= n_ops <= ION_MAX_HOPS
 *   operators (ops: a host array), one pass over g; a two-stage FP64 sum with a
 *   compensated second stage; scratch from ion_expectation_scratch_bytes.
 * ------------------------------------------------------------------------ */
enum { ION_HOP_IMAG_B = 1, ION_HOP_IMAG_A = 2, ION_HOP_WRAP_B = 4, ION_MAX_HOPS = 4 };
typedef struct ion_hop {
    const double *diag;  /* [n_a*n_b] or NULL */
    const double *off_b; /* [n_a*n_b]: coupling of (i, j) and (i, j+1) (j = n_b-1 unused), or NULL */
    const double *off_a; /* [n_a*n_b]: coupling of (i, j) and (i+1, j) (i = n_a-1 unused), or NULL */
    int32_t flags;       /* ION_HOP_IMAG_B | ION_HOP_IMAG_A | ION_HOP_WRAP_B */
    int32_t pad_;
} ion_hop;
int64_t ion_expectation_scratch_bytes(int32_t n_a, int32_t n_b, int32_t n_ops);
int ion_expectation_c128(const void *g, int32_t n_a, int32_t n_b, int32_t n_ops, const ion_hop *ops, double weight,
                         double *out, void *scratch, int64_t scratch_bytes, void *stream);
int ion_expectation_c64(const void *g, const void *g_lo, int32_t n_a, int32_t n_b, int32_t n_ops,
                        const ion_hop *ops, double weight, double *out, void *scratch, int64_t scratch_bytes,
                        void *stream);

/* The radial probability current of a spherical-harmonic mesh (the
 * DirectionalRadialProbabilityCurrent datastore, data.py:467-530, with
 * SphericalHarmonicMesh.get_radial_probability_current_density_mesh__spatial,
 * meshes.py:1358-1371, and the r-current operator of
 * SphericalHarmonicLengthGaugeOperators.r_probability_current__spatial,
 * mesh_operators.py:1107-1127), on (n_l, n_r) g:
 *   out[j] (z > 0) and out[n_r + j] (z < 0) =
 *     r[j]^2 Im(sum_{l,l'} conj(g[l][j]) W[l][l'] (od[j] g[l'][j+1] - od[j-1] g[l'][j-1]))
 * with W = w_pos or w_neg ([n_l*n_l], symmetric): 2 pi dtheta times the sum
 * over that hemisphere's theta points of sin(theta) Y_l(theta) Y_l'(theta),
 * and od [n_r-1] the operator's couplings.  out: device [2*n_r]. */
int ion_sh_radial_current_c128(const void *g, int32_t n_r, int32_t n_l, const double *od, const double *r,
                               const double *w_pos, const double *w_neg, double *out, void *stream);
int ion_sh_radial_current_c64(const void *g, const void *g_lo, int32_t n_r, int32_t n_l, const double *od,
                              const double *r, const double *w_pos, const double *w_neg, double *out,
                              void *stream);

#ifdef __cplusplus
}
#endif

#endif /* IONIZATION_GB300_H */
