// The optimize pass on caller-owned device buffers with no device allocation
// (ptl_optimize_noalloc in include/ptl_codegen.h).
//
// Who needs it: a caller that owns the device's memory budget outright -- a compile
// server that reserves one pool at start-up and admits requests against it, or an
// engine whose allocator must see every byte -- cannot let a library call cudaMalloc
// behind its back, and a cudaMalloc/cudaFree in the middle of a stream of work also
// synchronises the device.  Such a caller can still run this pass on buffers it
// already holds: its scratch (one liveness byte and one store-operand byte per word,
// a changed flag and an error word) lives in the fixed array below, which every GPU
// that loads this library holds until the process exits.
//
// The same per-word stage functions as the generator's optimize stage
// (rv_generator_avx.cpp:891-1016) run here; only the storage differs, and the loops stop
// at count instead of running over the generator's padded lanes (the padding lanes hold
// no virtual register, so they change nothing inside [0, count)).
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ptl_codegen.h"
#include "ptl_kernels.cuh"
#include "ptl_stages.cuh"

using namespace ptl;

namespace {

constexpr size_t kMaxWords = PTL_OPTIMIZE_NOALLOC_MAX_WORDS;
constexpr size_t kHeader = 256;  // ErrorWord at 0, changed flag at 64
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

// used[kMaxWords] then smark[kMaxWords] after the header: 8 MiB + 256 bytes.
static __device__ __align__(256) unsigned char g_opt_scratch[kHeader + 2 * kMaxWords];

struct DeviceScratch {
    std::once_flag once;
    unsigned char* base = nullptr;
    cudaError_t setup = cudaSuccess;
    std::mutex lock;  // one scratch area per device: calls on a device run one at a time
};
DeviceScratch g_scratch[kMaxDevices];

unsigned grid_of(size_t n) {
    size_t g = (n + kThreads - 1) / kThreads;
    if (g < 1) g = 1;
    if (g > 152u * 16u) g = 152u * 16u;  // grid-stride loops beyond 16 CTAs per SM
    return static_cast<unsigned>(g);
}

#define NOALLOC_FOR(i, count)                                                            \
    for (size_t i##_ = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;       \
         i##_ < (count); i##_ += static_cast<size_t>(gridDim.x) * blockDim.x)            \
        if (const uint32_t i = static_cast<uint32_t>(i##_); true)

__global__ void k_na_mark(Prog P) { NOALLOC_FOR(i, P.W) st_opt_mark(P, i); }

__global__ void k_na_sweep(Prog P) {
    bool any = false;
    NOALLOC_FOR(i, P.W) any |= st_opt_sweep(P, i);
    if (__syncthreads_or(any) && threadIdx.x == 0) P.flags[0] = 1;
}

__global__ void k_na_final(Prog P) { NOALLOC_FOR(i, P.W) st_opt_final(P, i); }

bool is_device_pointer(const void* p, int device) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) && a.device == device;
}

// Once work is queued on the caller's stream, every return waits for it: the lock that
// serialises calls on this device is released on return, and the next call (perhaps on
// another stream) reuses the scratch at once.
struct DrainOnReturn {
    cudaStream_t s;
    ~DrainOnReturn() {
        cudaStreamSynchronize(s);
        cudaGetLastError();
    }
};

ptl_status run(const uint32_t* instr, const uint32_t* rd, const uint32_t* rs1, const uint32_t* rs2,
               uint32_t count, uint32_t* used_instrs, cudaStream_t s, unsigned char* base) {
    DrainOnReturn drain{s};
    Prog P{};
    P.W = count;
    P.wb8 = count;
    P.instr = const_cast<uint32_t*>(instr);
    P.rd = const_cast<uint32_t*>(rd);
    P.rs1 = const_cast<uint32_t*>(rs1);
    P.rs2 = const_cast<uint32_t*>(rs2);
    P.used_instrs = used_instrs;
    P.err = reinterpret_cast<ErrorWord*>(base);
    P.flags = reinterpret_cast<uint32_t*>(base + 64);
    P.used = base + kHeader;
    P.smark = base + kHeader + kMaxWords;

    // what must start at zero: the error word, the flag and both mark arrays
    if (cudaMemsetAsync(base, 0, kHeader, s) != cudaSuccess) return PTL_CUDA_ERROR;
    if (cudaMemsetAsync(P.used, 0, count, s) != cudaSuccess) return PTL_CUDA_ERROR;
    if (cudaMemsetAsync(P.smark, 0, count, s) != cudaSuccess) return PTL_CUDA_ERROR;
    const unsigned grid = grid_of(count);
    note_launch();
    k_na_mark<<<grid, kThreads, 0, s>>>(P);
    for (uint32_t sweeps = 0;;) {
        if (cudaMemsetAsync(P.flags, 0, sizeof(uint32_t), s) != cudaSuccess) return PTL_CUDA_ERROR;
        for (int k = 0; k < 4; ++k) {
            note_launch();
            k_na_sweep<<<grid, kThreads, 0, s>>>(P);
        }
        sweeps += 4;
        uint32_t changed = 0;
        if (cudaMemcpyAsync(&changed, P.flags, sizeof(changed), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return PTL_CUDA_ERROR;
        if (!changed) break;
        if (sweeps > count + 8u) return PTL_DEVICE_TIMEOUT;  // every sweep that continues clears a mark
    }
    note_launch();
    k_na_final<<<grid, kThreads, 0, s>>>(P);
    ErrorWord e{};
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpyAsync(&e, P.err, sizeof(e), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PTL_CUDA_ERROR;
    return e.code == ST_OK ? PTL_OK : static_cast<ptl_status>(e.code);
}

}  // namespace

extern "C" ptl_status ptl_optimize_noalloc(const uint32_t* instr, const uint32_t* rd, const uint32_t* rs1,
                                           const uint32_t* rs2, size_t count, uint32_t* used_instrs,
                                           void* stream) {
    if (count > kMaxWords) return PTL_BAD_ARGUMENT;  // above PTL_OPTIMIZE_NOALLOC_MAX_WORDS
    if (count == 0) return PTL_OK;
    if (!instr || !rd || !rs1 || !rs2 || !used_instrs) return PTL_BAD_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return PTL_CUDA_ERROR;
    DeviceScratch& d = g_scratch[dev];
    // set-up, once per device, with that device current: the scratch array's address
    std::call_once(d.once, [&] {
        d.setup = cudaGetSymbolAddress(reinterpret_cast<void**>(&d.base), g_opt_scratch);
        if (d.setup != cudaSuccess) d.base = nullptr;
    });
    if (d.setup != cudaSuccess || !d.base) return PTL_CUDA_ERROR;
    for (const void* p : {static_cast<const void*>(instr), static_cast<const void*>(rd),
                          static_cast<const void*>(rs1), static_cast<const void*>(rs2),
                          static_cast<const void*>(used_instrs)}) {
        if (!is_device_pointer(p, dev)) return PTL_BAD_ARGUMENT;
    }
    // the call waits for its result on the host, which a capturing stream cannot do
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess) {
        cudaGetLastError();
        return PTL_BAD_ARGUMENT;
    }
    if (cap != cudaStreamCaptureStatusNone) return PTL_BAD_ARGUMENT;
    std::lock_guard<std::mutex> hold(d.lock);
    return run(instr, rd, rs1, rs2, static_cast<uint32_t>(count), used_instrs, static_cast<cudaStream_t>(stream),
               d.base);
}
