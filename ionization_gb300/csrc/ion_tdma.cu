// Thomas / tridiagonal solves: the drop-in for the reference's cy.tdma
// (ionization/cy.pyx:9-50, called from TDMAOperator._apply,
// ionization/mesh/mesh_operators.py:109-111).
//
//  * ion_tdma_batched_*: nsys systems of n rows, one CTA per system, solved by
//    the block partition + PCR solver of ion_solver.cuh.
//  * ion_tdma_*: one system of any length.  Up to one CTA's capacity it is the
//    same block solve; beyond that, a multi-level partition through global
//    scratch: level l splits its rows into chunks of <= MAXM rows (one thread
//    each), stores alpha/beta/gamma of every interior row in scratch and emits
//    a reduced system of 2 rows per chunk, which becomes level l+1; the last
//    level fits one CTA.  The expansion kernels then walk back down.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "ion_common.cuh"
#include "ion_solver.cuh"

namespace ion {

// per-precision tuning: rows per thread and largest CTA
template <typename R> struct TdmaCfg;
template <> struct TdmaCfg<double> {
    static constexpr int MAXM = 8;
    static constexpr int MAX_T = 512;
};
template <> struct TdmaCfg<float> {
    static constexpr int MAXM = 16;
    static constexpr int MAX_T = 512;
};

template <typename R>
static int64_t block_capacity() {
    return int64_t(TdmaCfg<R>::MAXM) * TdmaCfg<R>::MAX_T;
}

// threads for a one-CTA solve of n rows: ceil(n / MAXM), at most n/2
template <typename R>
static int block_threads(int64_t n) {
    int64_t T = (n + TdmaCfg<R>::MAXM - 1) / TdmaCfg<R>::MAXM;
    if (T > n / 2) T = n / 2;
    if (T < 1) T = 1;
    return int(T);
}

static int round_up32(int x) { return (x + 31) / 32 * 32; }

// ---------------------------------------------------------------------------
// coefficient / rhs / output functors
// ---------------------------------------------------------------------------
template <typename R>
struct DiaCoef {  // the reference's dia layout, rows [base, base+n)
    const Cx<R>* sub;
    const Cx<R>* diag;
    const Cx<R>* sup;
    int64_t base, n;
    __device__ void operator()(int64_t i, Cx<R>& a, Cx<R>& b, Cx<R>& c) const {
        const Cx<R> zero = {R(0), R(0)};
        a = (i > 0) ? ld(sub + base + i - 1) : zero;
        b = ld(diag + base + i);
        c = (i < n - 1) ? ld(sup + base + i) : zero;
    }
};

template <typename R>
struct RedCoef {  // a normalised reduced system: b = 1
    const Cx<R>* a_;
    const Cx<R>* c_;
    int64_t n;
    __device__ void operator()(int64_t i, Cx<R>& a, Cx<R>& b, Cx<R>& c) const {
        const Cx<R> zero = {R(0), R(0)};
        a = (i > 0) ? ld(a_ + i) : zero;
        b = Cx<R>{R(1), R(0)};
        c = (i < n - 1) ? ld(c_ + i) : zero;
    }
};

template <typename R>
struct VecRhs {
    const Cx<R>* v;
    int64_t base;
    __device__ Cx<R> operator()(int64_t i) const { return ld(v + base + i); }
};

template <typename R>
struct VecOut {
    Cx<R>* v;
    int64_t base;
    __device__ void operator()(int64_t i, Cx<R> x) const { st(v + base + i, x); }
};

// ---------------------------------------------------------------------------
// one CTA per system
// ---------------------------------------------------------------------------
template <typename R, int MAXM, class Coef, class Rhs, class Out>
__device__ __forceinline__ void block_solve_system(int64_t n, int T, const Coef& coef,
                                                   const Rhs& rhs, const Out& out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Cx<R>* red = reinterpret_cast<Cx<R>*>(smem_raw);
    const int t = threadIdx.x;
    block_line_solve<R, MAXM>(int(n), T, t, t < T, red, coef, rhs, out);
}

template <typename R, int MAXM>
__global__ void __launch_bounds__(512) tdma_batched_kernel(int64_t n, int T, const Cx<R>* sub,
                                                           const Cx<R>* diag, const Cx<R>* sup,
                                                           const Cx<R>* d, Cx<R>* x) {
    const int64_t base = int64_t(blockIdx.x) * n;
    DiaCoef<R> coef{sub, diag, sup, base, n};
    block_solve_system<R, MAXM>(n, T, coef, VecRhs<R>{d, base}, VecOut<R>{x, base});
}

template <typename R, int MAXM>
__global__ void __launch_bounds__(512) tdma_reduced_block_kernel(int64_t n, int T, const Cx<R>* ra,
                                                                 const Cx<R>* rc, const Cx<R>* rd,
                                                                 Cx<R>* x) {
    RedCoef<R> coef{ra, rc, n};
    block_solve_system<R, MAXM>(n, T, coef, VecRhs<R>{rd, 0}, VecOut<R>{x, 0});
}

// n == 1: x = d / b
template <typename R>
__global__ void tdma_single_row_kernel(const Cx<R>* diag, const Cx<R>* d, Cx<R>* x) {
    st(x, ld(d) * crecip(ld(diag)));
}

// ---------------------------------------------------------------------------
// multi-level partition through global scratch
// ---------------------------------------------------------------------------
template <typename R, int MAXM, class Coef, class Rhs>
__global__ void __launch_bounds__(256) partition_eliminate_kernel(int64_t n, int64_t P, Coef coef,
                                                                  Rhs rhs, Cx<R>* A, Cx<R>* B,
                                                                  Cx<R>* G, Cx<R>* ra, Cx<R>* rc,
                                                                  Cx<R>* rd) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= P) return;
    int64_t s;
    int m;
    chunk_bounds(n, P, t, s, m);
    Cx<R> al[MAXM], be[MAXM], ga[MAXM];
    RedRow<R> rS, rE;
    chunk_eliminate<R, MAXM>(s, m, coef, rhs, al, be, ga, rS, rE);
#pragma unroll
    for (int k = 1; k < MAXM - 1; ++k) {
        if (k <= m - 2) {
            st(A + s + k, al[k]);
            st(B + s + k, be[k]);
            st(G + s + k, ga[k]);
        }
    }
    st(ra + 2 * t, rS.a);
    st(rc + 2 * t, rS.c);
    st(rd + 2 * t, rS.d);
    st(ra + 2 * t + 1, rE.a);
    st(rc + 2 * t + 1, rE.c);
    st(rd + 2 * t + 1, rE.d);
}

template <typename R, int MAXM>
__global__ void __launch_bounds__(256) partition_expand_kernel(int64_t n, int64_t P, const Cx<R>* A,
                                                               const Cx<R>* B, const Cx<R>* G,
                                                               const Cx<R>* xred, Cx<R>* x) {
    const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= P) return;
    int64_t s;
    int m;
    chunk_bounds(n, P, t, s, m);
    const Cx<R> xs = ld(xred + 2 * t), xe = ld(xred + 2 * t + 1);
    st(x + s, xs);
    for (int k = 1; k <= m - 2; ++k) {
        const Cx<R> v = ld(A + s + k) + ld(B + s + k) * xs + ld(G + s + k) * xe;
        st(x + s + k, v);
    }
    st(x + s + m - 1, xe);
}

// level sizes: n_0 = n, n_{l+1} = 2 * P_l with P_l = ceil(n_l / MAXM), until
// n_l fits one CTA
template <typename R>
struct Levels {
    int count = 0;
    int64_t n[32];
    int64_t P[32];
};

template <typename R>
static Levels<R> plan_levels(int64_t n) {
    Levels<R> L;
    int64_t cur = n;
    while (cur > block_capacity<R>() && L.count < 31) {
        const int64_t P = (cur + TdmaCfg<R>::MAXM - 1) / TdmaCfg<R>::MAXM;
        L.n[L.count] = cur;
        L.P[L.count] = P;
        L.count++;
        cur = 2 * P;
    }
    L.n[L.count] = cur;  // final (one-CTA) level
    return L;
}

// scratch per partition level: A, B, G (n_l each) + ra, rc, rd, xred (2 P_l each)
template <typename R>
static int64_t scratch_elems(int64_t n) {
    Levels<R> L = plan_levels<R>(n);
    int64_t e = 0;
    for (int l = 0; l < L.count; ++l) e += 3 * L.n[l] + 4 * 2 * L.P[l];
    return e;
}

template <typename R>
static size_t block_smem(int T) {
    return pcr_smem_bytes<R>(T);
}

template <typename R, int MAXM, class K>
static int set_smem_attr(K kernel, size_t bytes) {
    (void)bytes;
    return ensure_smem_limit(reinterpret_cast<const void*>(kernel), 200 * 1024, "ion_tdma");
}

template <typename R>
static int tdma_impl(int64_t n, const void* sub, const void* diag, const void* sup, const void* d,
                     void* x, void* scratch, int64_t scratch_bytes, void* stream) {
    constexpr int MAXM = TdmaCfg<R>::MAXM;
    if (n < 1 || !diag || !d || !x || (n > 1 && (!sub || !sup))) {
        set_error("ion_tdma: invalid argument (n=%lld)", (long long)n);
        return ION_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t st_ = as_stream(stream);
    const Cx<R>* sub_ = static_cast<const Cx<R>*>(sub);
    const Cx<R>* diag_ = static_cast<const Cx<R>*>(diag);
    const Cx<R>* sup_ = static_cast<const Cx<R>*>(sup);
    const Cx<R>* d_ = static_cast<const Cx<R>*>(d);
    Cx<R>* x_ = static_cast<Cx<R>*>(x);
    if (n == 1) {
        tdma_single_row_kernel<R><<<1, 1, 0, st_>>>(diag_, d_, x_);
        return check_launch("tdma_single_row_kernel");
    }
    const int64_t need = scratch_elems<R>(n) * int64_t(sizeof(Cx<R>));
    if (need > 0 && (scratch == nullptr || scratch_bytes < need)) {
        set_error("ion_tdma: scratch too small (%lld bytes given, %lld needed)",
                  (long long)scratch_bytes, (long long)need);
        return ION_ERR_SCRATCH_TOO_SMALL;
    }
    Levels<R> L = plan_levels<R>(n);
    if (L.count == 0) {
        const int T = block_threads<R>(n);
        auto k = tdma_batched_kernel<R, MAXM>;
        if (int rc = set_smem_attr<R, MAXM>(k, block_smem<R>(T))) return rc;
        k<<<1, round_up32(T), block_smem<R>(T), st_>>>(n, T, sub_, diag_, sup_, d_, x_);
        return check_launch("tdma_batched_kernel");
    }
    // carve scratch
    Cx<R>* base = static_cast<Cx<R>*>(scratch);
    Cx<R>*A[32], *B[32], *G[32], *ra[32], *rc[32], *rd[32], *xr[32];
    for (int l = 0; l < L.count; ++l) {
        A[l] = base;
        base += L.n[l];
        B[l] = base;
        base += L.n[l];
        G[l] = base;
        base += L.n[l];
        ra[l] = base;
        base += 2 * L.P[l];
        rc[l] = base;
        base += 2 * L.P[l];
        rd[l] = base;
        base += 2 * L.P[l];
        xr[l] = base;
        base += 2 * L.P[l];
    }
    // eliminate downwards
    for (int l = 0; l < L.count; ++l) {
        const int64_t P = L.P[l];
        const int threads = 256;
        const int64_t blocks = (P + threads - 1) / threads;
        if (l == 0) {
            DiaCoef<R> coef{sub_, diag_, sup_, 0, n};
            partition_eliminate_kernel<R, MAXM><<<blocks, threads, 0, st_>>>(
                L.n[0], P, coef, VecRhs<R>{d_, 0}, A[0], B[0], G[0], ra[0], rc[0], rd[0]);
        } else {
            RedCoef<R> coef{ra[l - 1], rc[l - 1], L.n[l]};
            partition_eliminate_kernel<R, MAXM><<<blocks, threads, 0, st_>>>(
                L.n[l], P, coef, VecRhs<R>{rd[l - 1], 0}, A[l], B[l], G[l], ra[l], rc[l], rd[l]);
        }
        if (int e = check_launch("partition_eliminate_kernel")) return e;
    }
    // the last reduced system in one CTA
    {
        const int last = L.count - 1;
        const int64_t nf = L.n[L.count];
        const int T = block_threads<R>(nf);
        auto k = tdma_reduced_block_kernel<R, MAXM>;
        if (int rc_ = set_smem_attr<R, MAXM>(k, block_smem<R>(T))) return rc_;
        k<<<1, round_up32(T), block_smem<R>(T), st_>>>(nf, T, ra[last], rc[last], rd[last], xr[last]);
        if (int e = check_launch("tdma_reduced_block_kernel")) return e;
    }
    // expand upwards
    for (int l = L.count - 1; l >= 0; --l) {
        const int64_t P = L.P[l];
        const int threads = 256;
        const int64_t blocks = (P + threads - 1) / threads;
        Cx<R>* out = (l == 0) ? x_ : xr[l - 1];
        partition_expand_kernel<R, MAXM><<<blocks, threads, 0, st_>>>(L.n[l], P, A[l], B[l], G[l],
                                                                       xr[l], out);
        if (int e = check_launch("partition_expand_kernel")) return e;
    }
    return ION_OK;
}

template <typename R>
static int tdma_batched_impl(int64_t nsys, int64_t n, const void* sub, const void* diag,
                             const void* sup, const void* d, void* x, void* stream) {
    constexpr int MAXM = TdmaCfg<R>::MAXM;
    if (nsys < 0 || n < 2 || n > block_capacity<R>() || nsys > 2147483647LL || !sub || !diag ||
        !sup || !d || !x) {
        set_error("ion_tdma_batched: invalid argument (nsys=%lld, n=%lld, max n=%lld)",
                  (long long)nsys, (long long)n, (long long)block_capacity<R>());
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (nsys == 0) return ION_OK;
    const int T = block_threads<R>(n);
    auto k = tdma_batched_kernel<R, MAXM>;
    if (int rc = set_smem_attr<R, MAXM>(k, block_smem<R>(T))) return rc;
    k<<<unsigned(nsys), round_up32(T), block_smem<R>(T), as_stream(stream)>>>(
        n, T, static_cast<const Cx<R>*>(sub), static_cast<const Cx<R>*>(diag),
        static_cast<const Cx<R>*>(sup), static_cast<const Cx<R>*>(d), static_cast<Cx<R>*>(x));
    return check_launch("tdma_batched_kernel");
}

}  // namespace ion

// ---------------------------------------------------------------------------
// Scratch-free entry point: the single-system solve with its partition
// scratch in a fixed, file-scope device array rather than caller memory.
// ---------------------------------------------------------------------------
namespace ion {

// Largest system it accepts, and the scratch that size needs
// (ion_tdma_scratch_bytes_c128(65536); the need grows with n up to there).
constexpr int64_t NOALLOC_MAX_N = 65536;
constexpr int64_t NOALLOC_SCRATCH_BYTES = 5242880;

// Held by every GPU that loads this library, until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];

// The array's name is only a host-side stand-in; its device address belongs
// to the CUDA context that loaded this module.  It is looked up with the
// device current and cached per device together with that context's id, so a
// new context on the same device (after cudaDeviceReset, say) looks it up
// again instead of reusing a stale address.
struct NoallocSlot {
    unsigned long long ctx;
    void* addr;
};
static NoallocSlot g_noalloc_slot[64] = {};
static std::mutex g_noalloc_mu;

static int noalloc_scratch_address(cudaStream_t stream, void** out) {
    int dev = 0;
    unsigned long long ctx = 0;
    if (current_context(&dev, &ctx)) {
        set_error("ion_tdma_noalloc_c128: %s", last_error());
        return ION_ERR_CUDA;
    }
    if (dev < 0 || dev >= 64) {
        set_error("ion_tdma_noalloc_c128: device ordinal %d is beyond the 64 this library tracks", dev);
        return ION_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocSlot& slot = g_noalloc_slot[dev];
    if (slot.addr != nullptr && slot.ctx == ctx) {
        *out = slot.addr;
        return ION_OK;
    }
    // the lookup may load the module, which a stream capture does not allow
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        set_error("ion_tdma_noalloc_c128: the first call in this CUDA context on device %d is under stream "
                  "capture; call it once before capturing", dev);
        return ION_ERR_INVALID_ARGUMENT;
    }
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        set_error("ion_tdma_noalloc_c128: cudaGetSymbolAddress failed (%s)", cudaGetErrorString(e));
        return ION_ERR_CUDA;
    }
    slot.ctx = ctx;
    slot.addr = p;
    *out = p;
    return ION_OK;
}

static int tdma_noalloc_c128(int64_t n, const void* sub, const void* diag, const void* sup, const void* d,
                             void* x, void* stream) {
    if (n < 1 || n > NOALLOC_MAX_N) {
        set_error("ion_tdma_noalloc_c128: n = %lld is outside 1..%lld (the size of its fixed scratch)",
                  (long long)n, (long long)NOALLOC_MAX_N);
        return ION_ERR_INVALID_ARGUMENT;
    }
    const int64_t need = scratch_elems<double>(n) * int64_t(sizeof(Cx<double>));
    if (need > NOALLOC_SCRATCH_BYTES) {
        set_error("ion_tdma_noalloc_c128: n = %lld needs %lld scratch bytes, more than the %lld held",
                  (long long)n, (long long)need, (long long)NOALLOC_SCRATCH_BYTES);
        return ION_ERR_INVALID_ARGUMENT;
    }
    // looked up on every call, whatever n is, so that the first call in a
    // context does the set-up even when it is a small system
    void* scratch = nullptr;
    if (int e = noalloc_scratch_address(as_stream(stream), &scratch)) return e;
    // every scratch word the partition reads is written earlier in the same
    // call, so nothing has to be cleared between calls
    return tdma_impl<double>(n, sub, diag, sup, d, x, need > 0 ? scratch : nullptr, NOALLOC_SCRATCH_BYTES, stream);
}

}  // namespace ion

using namespace ion;

extern "C" {

int ion_tdma_noalloc_c128(int64_t n, const void* sub, const void* diag, const void* sup, const void* d, void* x,
                          void* stream) {
    return tdma_noalloc_c128(n, sub, diag, sup, d, x, stream);
}
int64_t ion_tdma_noalloc_max_n_c128(void) { return NOALLOC_MAX_N; }


int64_t ion_tdma_scratch_bytes_c128(int64_t n) {
    return n < 1 ? 0 : scratch_elems<double>(n) * int64_t(sizeof(Cx<double>));
}
int64_t ion_tdma_scratch_bytes_c64(int64_t n) {
    return n < 1 ? 0 : scratch_elems<float>(n) * int64_t(sizeof(Cx<float>));
}
int ion_tdma_c128(int64_t n, const void* sub, const void* diag, const void* sup, const void* d,
                  void* x, void* scratch, int64_t scratch_bytes, void* stream) {
    return tdma_impl<double>(n, sub, diag, sup, d, x, scratch, scratch_bytes, stream);
}
int ion_tdma_c64(int64_t n, const void* sub, const void* diag, const void* sup, const void* d,
                 void* x, void* scratch, int64_t scratch_bytes, void* stream) {
    return tdma_impl<float>(n, sub, diag, sup, d, x, scratch, scratch_bytes, stream);
}
int ion_tdma_batched_c128(int64_t nsys, int64_t n, const void* sub, const void* diag,
                          const void* sup, const void* d, void* x, void* stream) {
    return tdma_batched_impl<double>(nsys, n, sub, diag, sup, d, x, stream);
}
int ion_tdma_batched_c64(int64_t nsys, int64_t n, const void* sub, const void* diag,
                         const void* sup, const void* d, void* x, void* stream) {
    return tdma_batched_impl<float>(nsys, n, sub, diag, sup, d, x, stream);
}
int64_t ion_tdma_batched_max_n_c128(void) { return block_capacity<double>(); }
int64_t ion_tdma_batched_max_n_c64(void) { return block_capacity<float>(); }

}  // extern "C"
