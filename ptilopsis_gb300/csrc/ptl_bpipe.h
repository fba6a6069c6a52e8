// Batched pipeline: many programs through the seven stages with one launch per stage
// step (ptl_bpipe.cu).  Host-only interface (no CUDA types), used by ptl_batch.cpp.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

#include "../../include/ptl_codegen.h"

namespace ptl {

// One program's output: pointers into the pipeline's host buffers, valid until its next
// compile.
struct BatchResult {
    ptl_status status = PTL_OK;
    const uint32_t* words = nullptr;
    size_t count = 0;
    const uint32_t *starts = nullptr, *ends = nullptr, *sizes = nullptr, *ids = nullptr;
    size_t functions = 0;
    uint64_t nodes = 0, words_gen = 0, words_ra = 0;  // n, words after isn_gen and regalloc
};

class BatchPipeline {
public:
    // Device and pinned host memory are kept between calls and grow to the largest batch.
    // urgent: the pipeline's stream gets the device's highest stream priority.
    static BatchPipeline* create(int device, int host_threads, ptl_status* st, bool urgent = false);
    virtual ~BatchPipeline() = default;
    // Compiles count host trees; out[k] receives program k's output or its status.
    // Returns PTL_OK unless the batch as a whole failed (CUDA error, out of memory).
    virtual ptl_status compile(const ptl_ast_view* trees, size_t count, std::vector<BatchResult>& out) = 0;
    // Device time of the last compile per stage (the reference's seven CSV columns), ns.
    virtual void stage_ns(uint64_t ns[7]) const = 0;
    // Device time of the last compile from its inputs on the device to its outputs
    // complete (before the output copy), ns.
    virtual uint64_t device_ns() const = 0;
    // Device time of the last compile's depth sort (part of isn_gen), ns.
    virtual uint64_t depth_sort_ns() const = 0;
    // Host-to-device and device-to-host bytes of the last compile.
    virtual void copied_bytes(uint64_t* h2d, uint64_t* d2h) const = 0;
    // Host-side parts of the last compile, ns: gathering the inputs into pinned memory,
    // the input copy, the output copy (device-timed).
    virtual void host_ns(uint64_t ns[3]) const = 0;
    // Elements per tile of the element-wise stages and of the optimize sweeps; returns
    // false (and changes nothing) for sizes the kernels do not take.
    virtual bool set_tiles(uint32_t elem_tile, uint32_t sweep_tile) = 0;
    // The part of the device's resident blocks the persistent regalloc launch may take
    // (default 1); less leaves SMs to pipelines on other streams.
    virtual void set_regalloc_share(double share) = 0;
    // The scalar generator's semantics (rv_generator_st) for the following compiles.
    virtual void set_scalar(bool on) = 0;
    virtual void tiles(uint32_t out[2]) const = 0;
    // Detail of the last failure.
    virtual const char* last_error() const = 0;
    // Device memory the pipeline's arenas hold now, bytes.
    virtual uint64_t device_bytes() const = 0;
    // Frees the arenas (between compiles only); the next compile allocates them again.
    virtual void release_memory() = 0;
};

}  // namespace ptl
