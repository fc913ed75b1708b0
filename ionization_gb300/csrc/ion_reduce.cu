// Whole-mesh norm and inner products: QuantumMesh.inner_product / norm
// (ionization/mesh/meshes.py:195-217) feeding the Norm and InnerProducts
// datastores (ionization/mesh/data.py:189-260).
//
// Stage 1: a grid of 2 x 152 CTAs (one wave on GB300) accumulates FP64
// partial sums of |g|^2 and conj(s) g per CTA (grid-stride, coalesced loads).
// Stage 2: one CTA adds the per-CTA partials with Neumaier compensation and
// applies the inner-product multiplier.
#include "ion_common.cuh"

namespace ion {

constexpr int RED_BLOCKS = 304;
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double block_reduce(double v, double* sh) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x < 32) {
        r = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
        r = warp_sum(r);
    }
    return r;
}

template <typename R>
__global__ void __launch_bounds__(RED_THREADS) reduce_stage1(int64_t M, const Cx<R>* g, int ns,
                                                             const Cx<double>* states, double* part) {
    __shared__ double sh[32];
    const int nq = 1 + 2 * ns;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    double acc = 0.0;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < M; k += stride) {
        const Cx<R> x = ld(g + k);
        acc += double(x.re) * double(x.re) + double(x.im) * double(x.im);
    }
    double r = block_reduce(acc, sh);
    if (threadIdx.x == 0) part[int64_t(blockIdx.x) * nq] = r;
    for (int s = 0; s < ns; ++s) {
        const Cx<double>* sv = states + int64_t(s) * M;
        double re = 0.0, im = 0.0;
        for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < M; k += stride) {
            const Cx<R> x = ld(g + k);
            const Cx<double> a = ld(sv + k);
            re += a.re * double(x.re) + a.im * double(x.im);  // conj(a) * x
            im += a.re * double(x.im) - a.im * double(x.re);
        }
        const double tr = block_reduce(re, sh);
        const double ti = block_reduce(im, sh);
        if (threadIdx.x == 0) {
            part[int64_t(blockIdx.x) * nq + 1 + 2 * s] = tr;
            part[int64_t(blockIdx.x) * nq + 2 + 2 * s] = ti;
        }
    }
}

__global__ void reduce_stage2(int nblocks, int ns, const double* part, double weight, double* out_norm,
                              double* out_ip) {
    const int nq = 1 + 2 * ns;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
        double sum = 0.0, comp = 0.0;
        for (int b = 0; b < nblocks; ++b) {
            const double v = part[int64_t(b) * nq + q];
            const double t = sum + v;
            comp += (fabs(sum) >= fabs(v)) ? (sum - t) + v : (v - t) + sum;
            sum = t;
        }
        sum = (sum + comp) * weight;
        if (q == 0) {
            if (out_norm) *out_norm = sum;
        } else if (out_ip) {
            out_ip[q - 1] = sum;
        }
    }
}

template <typename R>
static int reduce_impl(int64_t M, const void* g, int32_t ns, const void* states, double weight,
                       double* out_norm, double* out_ip, void* partials, void* stream) {
    if (M < 1 || !g || ns < 0 || (ns > 0 && (!states || !out_ip)) || !partials) {
        set_error("ion_reduce: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    cudaStream_t s = as_stream(stream);
    int blocks = int((M + RED_THREADS - 1) / RED_THREADS);
    if (blocks > RED_BLOCKS) blocks = RED_BLOCKS;
    reduce_stage1<R><<<blocks, RED_THREADS, 0, s>>>(M, static_cast<const Cx<R>*>(g), ns,
                                                    static_cast<const Cx<double>*>(states),
                                                    static_cast<double*>(partials));
    if (int e = check_launch("reduce_stage1")) return e;
    reduce_stage2<<<1, 64, 0, s>>>(blocks, ns, static_cast<const double*>(partials), weight, out_norm, out_ip);
    return check_launch("reduce_stage2");
}

// psi of a complex64 state as complex128: hi + lo (lo, the stored residual
// packed as bf16x2, may be absent), each component one FP64 sum of two
// floats.  Memory-bound; coalesced 8- and 4-byte loads, 16-byte stores.
__global__ void __launch_bounds__(256) psi_to_c128_kernel(int64_t n, const Cx<float>* hi, const uint32_t* lo,
                                                          Cx<double>* out) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const Cx<float> h = hi[i];
        Cx<double> v = {double(h.re), double(h.im)};
        if (lo) {
            const Cx<float> l = lo_unpack(lo[i]);
            v = Cx<double>{v.re + double(l.re), v.im + double(l.im)};
        }
        out[i] = v;
    }
}

// complex128 psi into the complex64 hi (nearest) and, if lo, the packed
// residual of psi - hi (each component's difference is exact in FP64 and
// rounded to FP32, then to bf16)
__global__ void __launch_bounds__(256) psi_split_kernel(int64_t n, const Cx<double>* in, Cx<float>* hi,
                                                        uint32_t* lo) {
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x) {
        const Cx<double> v = in[i];
        const Cx<float> h = {float(v.re), float(v.im)};
        hi[i] = h;
        if (lo) lo[i] = lo_pack(Cx<float>{float(v.re - double(h.re)), float(v.im - double(h.im))});
    }
}

// many rows, one CTA at a time per row (rows of a batch's initial states are
// a few thousand points each): split into hi and lo as psi_split_kernel, or
// copied into a complex128 hi
__global__ void __launch_bounds__(256) psi_split_rows_kernel(int64_t n_rows, const ion_psi_row* rows,
                                                             int hi_c128) {
    for (int64_t r = blockIdx.x; r < n_rows; r += gridDim.x) {
        const ion_psi_row row = rows[r];
        if (row.n <= 0 || !row.in || !row.hi) continue;  // an empty or NULL row writes nothing
        const Cx<double>* in = static_cast<const Cx<double>*>(row.in);
        if (hi_c128) {
            Cx<double>* out = static_cast<Cx<double>*>(row.hi);
            for (int64_t i = threadIdx.x; i < row.n; i += blockDim.x) out[i] = in[i];
            continue;
        }
        Cx<float>* hi = static_cast<Cx<float>*>(row.hi);
        uint32_t* lo = static_cast<uint32_t*>(row.lo);
        for (int64_t i = threadIdx.x; i < row.n; i += blockDim.x) {
            const Cx<double> v = in[i];
            const Cx<float> h = {float(v.re), float(v.im)};
            hi[i] = h;
            if (lo) lo[i] = lo_pack(Cx<float>{float(v.re - double(h.re)), float(v.im - double(h.im))});
        }
    }
}

}  // namespace ion

using namespace ion;

extern "C" {
int ion_psi_split_c128(int64_t n, const void* in, void* hi, void* lo, void* stream) {
    if (n < 0 || (n > 0 && (!in || !hi))) {
        set_error("ion_psi_split_c128: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return ION_OK;
    const int64_t want = (n + 255) / 256;
    const int blocks = int(want < 8 * 152 ? want : 8 * 152);
    psi_split_kernel<<<blocks, 256, 0, as_stream(stream)>>>(n, static_cast<const Cx<double>*>(in),
                                                             static_cast<Cx<float>*>(hi), static_cast<uint32_t*>(lo));
    return check_launch("psi_split_kernel");
}
int ion_psi_split_rows_c128(int64_t n_rows, const ion_psi_row* rows, int32_t hi_c128, void* stream) {
    if (n_rows < 0 || (n_rows > 0 && !rows)) {
        set_error("ion_psi_split_rows_c128: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (n_rows == 0) return ION_OK;
    const int blocks = int(n_rows < 16 * 152 ? n_rows : 16 * 152);
    psi_split_rows_kernel<<<blocks, 256, 0, as_stream(stream)>>>(n_rows, rows, hi_c128 ? 1 : 0);
    return check_launch("psi_split_rows_kernel");
}
int64_t ion_reduce_scratch_bytes(int64_t M, int32_t n_states) {
    (void)M;
    return int64_t(RED_BLOCKS) * (1 + 2 * int64_t(n_states < 0 ? 0 : n_states)) * int64_t(sizeof(double));
}
int ion_reduce_c128(int64_t M, const void* g, int32_t n_states, const void* states, double weight,
                    double* out_norm, double* out_ip, void* partials, void* stream) {
    return reduce_impl<double>(M, g, n_states, states, weight, out_norm, out_ip, partials, stream);
}
int ion_reduce_c64(int64_t M, const void* g, int32_t n_states, const void* states, double weight,
                   double* out_norm, double* out_ip, void* partials, void* stream) {
    return reduce_impl<float>(M, g, n_states, states, weight, out_norm, out_ip, partials, stream);
}
int ion_psi_to_c128(int64_t n, const void* hi, const void* lo, void* out, void* stream) {
    if (n < 0 || (n > 0 && (!hi || !out))) {
        set_error("ion_psi_to_c128: invalid argument");
        return ION_ERR_INVALID_ARGUMENT;
    }
    if (n == 0) return ION_OK;
    const int64_t want = (n + 255) / 256;
    const int blocks = int(want < 8 * 152 ? want : 8 * 152);
    psi_to_c128_kernel<<<blocks, 256, 0, as_stream(stream)>>>(n, static_cast<const Cx<float>*>(hi),
                                                               static_cast<const uint32_t*>(lo),
                                                               static_cast<Cx<double>*>(out));
    return check_launch("psi_to_c128_kernel");
}
}
