// Host-side runtime state shared by every translation unit of the library:
// the per-thread error string, launch checks, and settings that belong to a
// CUDA context rather than to the process (a kernel's dynamic shared-memory
// limit, a symbol's device address).  A process may drive several GPUs, and
// cudaDeviceReset replaces a device's context, so such settings are keyed on
// (device ordinal, context id) and redone when the context changes.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdarg>
#include <cstdio>
#include <map>
#include <mutex>
#include <utility>

#include "ion_common.cuh"

namespace ion {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

const char* last_error() { return g_err; }

int check_launch(const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("%s: %s", what, cudaGetErrorString(e));
        return ION_ERR_CUDA;
    }
    return ION_OK;
}

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points, so
// the library links only the runtime
static PFN_cuCtxGetCurrent_v4000 p_ctx_current = nullptr;
static PFN_cuCtxGetId_v12000 p_ctx_id = nullptr;
static std::once_flag g_entry_once;

static void load_entry_points() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        p_ctx_current = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        p_ctx_id = reinterpret_cast<PFN_cuCtxGetId_v12000>(f);
    cudaGetLastError();
}

int current_context(int* dev, unsigned long long* ctx_id) {
    std::call_once(g_entry_once, load_entry_points);
    cudaError_t e = cudaGetDevice(dev);
    if (e != cudaSuccess) {
        set_error("no usable CUDA device (%s)", cudaGetErrorString(e));
        return ION_ERR_CUDA;
    }
    if (!p_ctx_current || !p_ctx_id) {
        set_error("the CUDA driver lacks cuCtxGetCurrent / cuCtxGetId");
        return ION_ERR_CUDA;
    }
    CUcontext c = nullptr;
    if (p_ctx_current(&c) != CUDA_SUCCESS || c == nullptr) {
        // the runtime has not made the device's primary context current on
        // this thread yet; cudaSetDevice does that without allocating
        e = cudaSetDevice(*dev);
        if (e != cudaSuccess || p_ctx_current(&c) != CUDA_SUCCESS || c == nullptr) {
            set_error("no current CUDA context on device %d", *dev);
            return ION_ERR_CUDA;
        }
    }
    if (p_ctx_id(c, ctx_id) != CUDA_SUCCESS) {
        set_error("cuCtxGetId failed on device %d", *dev);
        return ION_ERR_CUDA;
    }
    return ION_OK;
}

// (kernel, device) -> (context id, limit set there)
static std::mutex g_smem_mu;
static std::map<std::pair<const void*, int>, std::pair<unsigned long long, int>> g_smem;

int ensure_smem_limit(const void* kernel, int bytes, const char* name) {
    int dev = 0;
    unsigned long long ctx = 0;
    if (int e = current_context(&dev, &ctx)) return e;
    std::lock_guard<std::mutex> lock(g_smem_mu);
    auto key = std::make_pair(kernel, dev);
    auto it = g_smem.find(key);
    if (it != g_smem.end() && it->second.first == ctx && it->second.second >= bytes) return ION_OK;
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_error("%s: cudaFuncSetAttribute(%d bytes of shared memory): %s", name, bytes, cudaGetErrorString(e));
        return ION_ERR_CUDA;
    }
    g_smem[key] = std::make_pair(ctx, bytes);
    return ION_OK;
}

// (device, caller's stream) -> (context id, side streams and events made for
// that stream).  Each caller stream has its own set, so launches issued on
// different streams (from one host thread or several) never share a side
// stream or an event: no false ordering between them, and a fork event is
// never re-recorded by another stream between its record and its waits.
static std::mutex g_fj_mu;
static std::map<std::pair<int, cudaStream_t>, std::pair<unsigned long long, ForkJoin*>> g_fj;
static constexpr int kMaxForkJoinPerDevice = 64;

ForkJoin* fork_join(cudaStream_t main) {
    int dev = 0;
    unsigned long long ctx = 0;
    if (current_context(&dev, &ctx)) return nullptr;
    std::lock_guard<std::mutex> lock(g_fj_mu);
    const auto key = std::make_pair(dev, main);
    auto it = g_fj.find(key);
    if (it != g_fj.end() && it->second.first == ctx) return it->second.second;
    // none for this stream in this context yet: make them, but not while the
    // stream is being captured (the caller then runs its launches in stream
    // order); handles of an earlier context went with it and are left alone
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(main, &st) != cudaSuccess || st != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return nullptr;
    }
    if (it == g_fj.end()) {
        int n = 0;
        for (const auto& e : g_fj) n += e.first.first == dev;
        if (n >= kMaxForkJoinPerDevice) return nullptr;  // many caller streams: stream order
    }
    // side streams at the caller's priority, so a high-priority caller's
    // work keeps its place in the block scheduler
    int prio = 0;
    if (cudaStreamGetPriority(main, &prio) != cudaSuccess) {
        cudaGetLastError();
        prio = 0;
    }
    auto* fj = new ForkJoin{};
    bool ok = cudaEventCreateWithFlags(&fj->fork, cudaEventDisableTiming) == cudaSuccess;
    for (int k = 0; ok && k < ForkJoin::N; ++k)
        ok = cudaStreamCreateWithPriority(&fj->s[k], cudaStreamNonBlocking, prio) == cudaSuccess &&
             cudaEventCreateWithFlags(&fj->join[k], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        cudaGetLastError();
        return nullptr;  // (what was made stays allocated; this is not retried in a loop)
    }
    g_fj[key] = std::make_pair(ctx, fj);
    return fj;
}

}  // namespace ion

extern "C" {
const char* ion_last_error(void) { return ion::last_error(); }
int ion_version(void) { return 101; }
}
