/*
 * ptilopsis_gb300 -- GB300 (sm_103a) implementation of Ptilopsis's data-parallel RISC-V
 * code generator, behind a plain C ABI.
 *
 * The reference's interface is the C++ class rv_generator_avx
 * (include/codegen/rv_generator_avx.hpp:58, src/codegen/rv_generator_avx.cpp:21-120 of
 * the reference): construct it from a DepthTree (the flattened post-order AST of
 * pareas-ast, subprojects/pareas-ast/include/codegen/depthtree.hpp:12-59), call
 * process(profile) (include/codegen/rv_generator.hpp:67), read get_instructions()
 * (src/codegen/rv_generator_avx.cpp:82-84) and, through the protected members
 * func_starts/func_ends/function_sizes/function_ids (include/codegen/rv_generator.hpp:
 * 46-51), the function table.  Each entry point below names the call it replaces.
 *
 * Output is bit-identical to the reference's one-worker-thread run of that class.
 * Errors are status codes; no C++ exception crosses this boundary.  A generator is not
 * thread-safe; distinct generators may be used from distinct threads.
 */
#ifndef PTL_CODEGEN_H
#define PTL_CODEGEN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    PTL_OK = 0,
    PTL_INVALID_AST = 1,        /* the arrays violate the DepthTree contract */
    PTL_UNSUPPORTED = 2,        /* input reaches behaviour the reference leaves undefined */
    PTL_OOM = 3,                /* device memory exhausted */
    PTL_ADMISSION_DENIED = 4,   /* a compile server refused the request (memory budget) */
    PTL_DEVICE_TIMEOUT = 5,     /* a bounded device-side wait gave up */
    PTL_CUDA_ERROR = 6,
    PTL_BAD_ARGUMENT = 7
} ptl_status;

/* A DepthTree: six parallel arrays of n nodes in post-order (children before parents,
 * the root last with parent -1 and child index -1).  type is the Pareas NodeType
 * (astnode.hpp:11-56), rtype the Pareas DataType (datatype.hpp:7-14).  With on_device
 * != 0 the pointers are CUDA device pointers on the generator's device. */
typedef struct {
    size_t n;
    size_t max_depth;
    const uint8_t* type;
    const uint8_t* rtype;
    const int32_t* parent;
    const int32_t* depth;
    const int32_t* child_idx;
    const uint32_t* data;
    int on_device;
} ptl_ast_view;

typedef struct ptl_generator ptl_generator;

/* Replaces rv_generator_avx(const DepthTree&, concurrency, sync, altblock, mininstr)
 * (rv_generator_avx.hpp:58): copies the tree to the device.  The scheduling arguments
 * of the CPU constructor have no GPU meaning and are not taken. */
ptl_status ptl_generator_create(const ptl_ast_view* tree, int device, ptl_generator** out);

/* Replaces the generator's input with another tree of any size, reusing the device
 * memory of earlier compiles (the reference builds a new generator per tree).  A host
 * tree is on the device when the call returns, so its arrays may be reused; a device
 * tree is copied on the generator's stream. */
ptl_status ptl_generator_upload(ptl_generator* gen, const ptl_ast_view* tree);

/* Replaces the scalar generator's constructor, rv_generator_st(const DepthTree&)
 * (include/codegen/rv_generator.hpp:82-84; main.cpp:123-124 picks it for -s): the same
 * generator object, whose process runs the single-threaded proof of concept's stages
 * (src/codegen/rv_generator.cpp:129-1736) instead of rv_generator_avx's.  Its output
 * differs from the AVX generator's (argument placement, float comparisons, isn_gen's
 * parent slots and jump targets, per-function register state and preserved registers)
 * and is bit-identical to rv_generator_st's.  Every other call below applies unchanged. */
ptl_status ptl_generator_create_scalar(const ptl_ast_view* tree, int device, ptl_generator** out);

/* Replaces rv_generator_avx::process(bool profile) (rv_generator_avx.cpp:104-120): runs
 * the seven stages.  Unlike the reference, which mutates its arrays and cannot be run
 * twice, process may be called again and recompiles from the copied tree.
 * profile bits: 1 = per-stage device times (ptl_generator_stage_ns); 2 = leave the words
 * on the device (ptl_generator_device_instructions); 4 = the register allocator finds
 * row-0 values through its hash table even when every virtual register has one
 * definition (the general path, normally taken only when one has two; same output);
 * 8 = a scalar generator allocates registers in the reference's serial order for every
 * program (normally only for programs whose functions name each other's words; same
 * output). */
ptl_status ptl_generator_process(ptl_generator* gen, int profile);

/* Replaces get_instructions() (rv_generator_avx.cpp:82-84): the encoded RV words, in a
 * host buffer owned by the generator, valid until the next process or destroy. */
ptl_status ptl_generator_instructions(ptl_generator* gen, const uint32_t** words, size_t* count);

/* The same words copied into the caller's buffer: dst null (or capacity too small, then
 * PTL_BAD_ARGUMENT) only sets *count.  After a process that left the words on the device
 * (flag 2) they go straight from the device into dst, without the generator's own copy;
 * into pageable memory whose pages the host has not touched yet that is slower than the
 * generator's copy, whose buffer keeps its pages from call to call. */
ptl_status ptl_generator_copy_instructions(ptl_generator* gen, uint32_t* dst, size_t capacity, size_t* count);

/* The same words as a device pointer (no copy). */
ptl_status ptl_generator_device_instructions(ptl_generator* gen, const uint32_t** words, size_t* count);

/* The function table the reference keeps in func_starts, func_ends, function_sizes and
 * function_ids (rv_generator.hpp:46-51), after its final fix_func_tab
 * (rv_generator_avx.cpp:1992).  Host buffers owned by the generator. */
ptl_status ptl_generator_function_table(ptl_generator* gen, const uint32_t** starts,
                                        const uint32_t** ends, const uint32_t** sizes,
                                        const uint32_t** ids, size_t* count);

/* Per-stage device time of the last process(profile != 0), in the order of the
 * reference's -p CSV (rv_generator.cpp:142-162): preprocess, isn_cnt, isn_gen,
 * optimize, regalloc, fix_jumps, postprocess (the last is fused into fix_jumps and
 * reported as 0). */
ptl_status ptl_generator_stage_ns(ptl_generator* gen, uint64_t ns[7]);

/* isn_gen's depth order on its own: pos[i] = the position of i in the order libstdc++'s
 * std::sort leaves iota(n) in when it sorts by keys[i] (the reference's isn_gen sort,
 * src/codegen/rv_generator_avx.cpp:539-541), computed by the GPU's emulation of that
 * introsort -- the order the generator uses to break ties between writers of a word.
 * keys are non-negative (depths).  For tests and tools; blocks until done. */
ptl_status ptl_depth_order(const int32_t* keys, size_t n, uint32_t* pos, int device);

/* Human-readable detail of the last non-OK status. */
const char* ptl_generator_last_error(const ptl_generator* gen);

void ptl_generator_destroy(ptl_generator* gen);

/* One-shot compile of a host tree into a caller buffer.  With words == NULL or a too
 * small capacity, *count receives the required size and PTL_BAD_ARGUMENT is returned
 * when words was given. */
ptl_status ptl_compile(const ptl_ast_view* tree, int device, uint32_t* words, size_t capacity,
                       size_t* count);

/* Intermediate arrays of the last process, for stage-by-stage parity checks.  which
 * selects the same arrays, in the same order, as the reference generator's members
 * after each stage (see ptilopsis_gb300/codegen.py SNAPSHOTS). */
ptl_status ptl_generator_snapshot(ptl_generator* gen, int which, uint32_t* out, size_t capacity,
                                  size_t* count);

/* The code tables in the reference's flat layouts (rv_nodetype.hpp:197-1134):
 * which = 0 node_size[256][6], 1 has_instr[256][4][6], 2 has_output[256][4][6],
 * 3 parent_arg_idx[256][4][6], 4 get_output[256][4][6], 5 instr[256][4][6],
 * 6 instr_constant[256][4], 7 operand[256][4][6][2], 8 instr_jt[256][4],
 * 9 pareas_to_rv[44].  Returns the element count; out may be NULL. */
size_t ptl_code_table(int which, uint32_t* out);

/* No counterpart in the reference: its optimize pass (rv_generator_avx.cpp:891-1016) runs
 * only inside process().  This is the same pass over caller-owned device buffers that
 * allocates no device memory, for callers that cannot have a library call cudaMalloc:
 * one that reserves the device's memory budget in its own pool and admits work against
 * it, or one that cannot take the device-wide synchronisation of a cudaMalloc/cudaFree
 * in the middle of its stream.  Its scratch is a fixed 8 MiB + 256 B array in device
 * memory that every GPU loading this library holds until the process exits.
 *
 * instr, rd, rs1, rs2: the count words of an isn_gen instruction stream and their
 * registers (the arrays ptl_generator_snapshot returns for which = 14..17), device
 * pointers on the current device.  used_instrs receives count words: 0xFFFFFFFF for a
 * word that stays, 0 for one the pass removes (ptl_generator_snapshot's which = 19).
 * stream is a cudaStream_t (NULL = the legacy default stream); the call blocks the
 * host until the result is written (it reads a changed flag back between sweeps), so a
 * stream that is being captured gets PTL_BAD_ARGUMENT with nothing queued on it.
 * count > PTL_OPTIMIZE_NOALLOC_MAX_WORDS returns PTL_BAD_ARGUMENT before touching
 * anything, as do null or non-device pointers.  The first call on each device looks up
 * the scratch array's address with that device current (cudaGetSymbolAddress); make
 * that first call before any stream capture begins.  Calls on one device are
 * serialised by a lock because they share the scratch, and every return, failures
 * included, comes after the call's device work has finished; device work that used the
 * same scratch concurrently would race. */
#define PTL_OPTIMIZE_NOALLOC_MAX_WORDS (1u << 22)
ptl_status ptl_optimize_noalloc(const uint32_t* instr, const uint32_t* rd, const uint32_t* rs1,
                                const uint32_t* rs2, size_t count, uint32_t* used_instrs, void* stream);

/* ---- Batched compilation.  No counterpart in the reference, which compiles one tree per
 * process (src/main.cpp:121-157).  All programs of a call go through the seven stages
 * together: one launch per stage step for the whole batch, per-program arrays in shared
 * device arenas kept between calls, sizes read back once per batch.  `workers` host
 * threads gather the inputs.  Each program's output is identical to compiling it alone;
 * a program that fails a check fails alone. */
typedef struct ptl_batch ptl_batch;
ptl_status ptl_batch_create(int device, int workers, ptl_batch** out);
/* Compiles count host trees; blocks until all are done.  Returns a batch-wide failure
 * (ptl_batch_last_error says which) or else the first program's non-OK status; each
 * program's own status is ptl_batch_status.  Results stay valid until the next compile. */
ptl_status ptl_batch_compile(ptl_batch* batch, const ptl_ast_view* trees, size_t count);
ptl_status ptl_batch_status(const ptl_batch* batch, size_t k);
ptl_status ptl_batch_words(const ptl_batch* batch, size_t k, const uint32_t** words, size_t* count);
ptl_status ptl_batch_function_table(const ptl_batch* batch, size_t k, const uint32_t** starts,
                                    const uint32_t** ends, const uint32_t** sizes, const uint32_t** ids,
                                    size_t* count);
/* Program k's node count and its word counts after isn_gen, regalloc and fix_jumps. */
ptl_status ptl_batch_sizes(const ptl_batch* batch, size_t k, uint64_t sizes[4]);
/* Wall time of the last ptl_batch_compile, in ns. */
uint64_t ptl_batch_elapsed_ns(const ptl_batch* batch);
/* Device time per stage of the last compile (ptl_generator_stage_ns's seven columns). */
ptl_status ptl_batch_stage_ns(const ptl_batch* batch, uint64_t ns[7]);
/* Device time of the last compile from its inputs on the device to its outputs complete
 * (before the output copy), in ns. */
uint64_t ptl_batch_device_ns(const ptl_batch* batch);
/* Device time of the last compile's depth sort (isn_gen's ordering of nodes by depth,
 * rv_generator_avx.cpp:526-566), in ns: the part of the isn_gen stage time that goes to
 * the sort rather than to the instruction writes. */
uint64_t ptl_batch_depth_sort_ns(const ptl_batch* batch);
/* Bytes copied host-to-device and device-to-host by the last compile. */
ptl_status ptl_batch_copied_bytes(const ptl_batch* batch, uint64_t* h2d, uint64_t* d2h);
/* Detail of the last batch-wide failure. */
const char* ptl_batch_last_error(const ptl_batch* batch);
/* Host-side parts of the last compile, ns: gathering the inputs into pinned memory, the
 * input copy and the output copy (both device-timed). */
ptl_status ptl_batch_host_ns(const ptl_batch* batch, uint64_t ns[3]);
/* Elements per tile of the batched element-wise stages (a power of two, 256..65536) and of
 * the optimize sweeps (512, 1024 or 2048); defaults 1024 and 1024.  No reference
 * counterpart: the reference's -i flag (minimum work per thread) is its nearest knob.
 * ptilopsis_gb300.batch.autotune measures the candidates and caches the choice. */
ptl_status ptl_batch_set_tiles(ptl_batch* batch, uint32_t elem_tile, uint32_t sweep_tile);
ptl_status ptl_batch_tiles(const ptl_batch* batch, uint32_t tiles[2]);
/* The part (0, 1] of the device's resident blocks the persistent register-allocation
 * launch may take (default 1).  Batches compiled at the same time on other handles of the
 * same device run beside it when it takes less. */
ptl_status ptl_batch_set_regalloc_share(ptl_batch* batch, double share);
/* scalar != 0: the following compiles give every program the scalar generator's output
 * (rv_generator_st, the reference's -s; ptl_generator_create_scalar one program at a
 * time); 0 (the default): the AVX generator's. */
ptl_status ptl_batch_set_scalar(ptl_batch* batch, int scalar);
void ptl_batch_destroy(ptl_batch* batch);

/* ---- AST flattening.  ptl_flatten replaces DepthTree::DepthTree(ASTNode*)
 * (pareas-ast/src/codegen/depthtree.cpp:11-100, the pointer-tree walk at :52-100) on the
 * GPU.  The reference walks the parser's pointer tree; a pointer tree does not cross to a
 * device, so the input is that tree as arrays in any node order: node v's parent is
 * parent[v] (-1 for the one root) and its place among its parent's children is
 * child_idx[v] (0 .. children-1).  The output is the DepthTree the reference builds: the
 * nodes in post-order (children in child_idx order before their parent), depth from the
 * root, parents as post-order indices, the root's child index -1 (the reference's
 * SIZE_MAX), and max_depth; order[v] (optional) receives v's post-order index.  Arrays
 * that are not one tree with child indices 0 .. k-1 (two roots or none, a parent out of
 * range, a child index out of range or taken twice, nodes the root does not reach) give
 * PTL_INVALID_AST.  Inputs and outputs are host arrays unless on_device; n < 2^31. */
typedef struct {
    size_t n;
    const uint8_t* type;
    const uint8_t* rtype;
    const int32_t* parent;
    const int32_t* child_idx;
    const uint32_t* data;
    int on_device;
} ptl_tree_view;

typedef struct {
    uint8_t* type;
    uint8_t* rtype;
    int32_t* parent;
    int32_t* depth;
    int32_t* child_idx;
    uint32_t* data;
    int32_t* order;    /* may be null */
    size_t max_depth;  /* written */
    int on_device;
} ptl_depth_tree_out;

/* stream: a cudaStream_t (null: the default stream).  Blocks until the result is ready. */
ptl_status ptl_flatten(const ptl_tree_view* in, ptl_depth_tree_out* out, int device, void* stream);

/* ---- Text output.  ptl_to_asm replaces rv_generator::to_asm
 * (src/codegen/rv_generator.cpp:121-127): one line per word, "name operands\n", as
 * rvdisasm::instruction prints it.  ptl_disassemble replaces rvdisasm::disassemble
 * (src/disassembler.cpp:411-451): the coloured listing with indices, addresses, bytes and
 * "funcN:" labels at the word indices in func_starts (n > 0).  Both write at most cap
 * bytes to out and set *len to the text's full length; out = NULL only measures. */
ptl_status ptl_to_asm(const uint32_t* words, size_t n, char* out, size_t cap, size_t* len);
ptl_status ptl_disassemble(const uint32_t* words, size_t n, uint64_t start_addr, const uint64_t* func_starts,
                           size_t nfunc, char* out, size_t cap, size_t* len);

/* ---- Object output.  No counterpart in the reference, which writes the raw words only
 * (rv_generator::to_binary, src/codegen/rv_generator.cpp:116-119).  Wraps the words and
 * the function table (ptl_generator_function_table's starts and ends, in words, in
 * address order) into an ELF64 little-endian RISC-V relocatable object: .text holds the
 * words, and each function is a global STT_FUNC symbol "funcN" (N = its position in the
 * table, the labels of ptl_disassemble) with value start*4 and size (end-start)*4.  The
 * generator's jumps are pc-relative within the program, so there are no relocations.
 * Writes the object to out (capacity bytes) and its size to *size; out = NULL only
 * measures.  PTL_BAD_ARGUMENT for a table that is not in address order or runs past the
 * words, or a capacity below the size. */
ptl_status ptl_write_elf(const uint32_t* words, size_t n_words, const uint32_t* func_starts,
                         const uint32_t* func_ends, size_t n_funcs, uint8_t* out, size_t capacity, size_t* size);

/* ---- Compile server.  No counterpart in the reference.  Continuous batching over
 * `slots` lanes (1..16), each a batched pipeline with its own stream and resident arenas:
 * a free lane takes every queued request of its size class (below or above 64k nodes;
 * with two or more lanes the first half takes only small requests, the others large ones
 * and small ones when no large one is queued), in arrival order, while the batch's
 * device-memory estimate fits in what is left of memory_budget (a later request that fits
 * may pass one that does not; at most 64M nodes per batch) and compiles them together,
 * while requests that arrive meanwhile go to the next free lane, so their work overlaps on
 * the GPU.  memory_budget bounds the device memory the lanes hold: each lane is charged
 * the larger of its resident arenas and its batch's estimate, idle lanes free their
 * arenas when a queued request needs the memory (ptl_server_memory).  Results are
 * identical to compiling each tree alone. */
typedef struct ptl_server ptl_server;
ptl_status ptl_server_create(int device, int slots, uint64_t memory_budget, ptl_server** out);
/* Copies a host tree into a request and queues it; PTL_ADMISSION_DENIED when the request
 * alone exceeds the budget. */
ptl_status ptl_server_submit(ptl_server* server, const ptl_ast_view* tree, uint64_t* ticket);
/* As ptl_server_submit; with PTL_SUBMIT_BORROW the request refers to the caller's arrays
 * instead of copying them (submit costs O(1)), and the caller keeps them alive and
 * unchanged until ptl_server_release of the ticket. */
#define PTL_SUBMIT_BORROW 1u
/* The request gets the scalar generator's output (rv_generator_st, the reference's -s);
 * a batch holds requests of one kind only. */
#define PTL_SUBMIT_SCALAR 2u
ptl_status ptl_server_submit_flags(ptl_server* server, const ptl_ast_view* tree, uint32_t flags, uint64_t* ticket);
/* *done = 1 once the request finished (wait != 0 blocks until then); returns its status. */
ptl_status ptl_server_poll(ptl_server* server, uint64_t ticket, int wait, int* done);
/* Output of a finished request (the table pointers may be NULL); valid until release. */
ptl_status ptl_server_result(ptl_server* server, uint64_t ticket, const uint32_t** words, size_t* count,
                             const uint32_t** starts, const uint32_t** ends, const uint32_t** sizes,
                             const uint32_t** ids, size_t* functions);
/* Submit, start and completion times of a finished request (ptl_clock_ns clock). */
ptl_status ptl_server_times(ptl_server* server, uint64_t ticket, uint64_t times[3]);
ptl_status ptl_server_release(ptl_server* server, uint64_t ticket);
/* Detail of a finished ticket's batch-wide failure (CUDA_ERROR, OOM); "" otherwise.
 * Valid until the ticket is released. */
const char* ptl_server_error(ptl_server* server, uint64_t ticket);
/* stats[0..4]: requests completed, nodes compiled, requests queued, admitted bytes in
 * flight, batches compiled. */
ptl_status ptl_server_stats(ptl_server* server, uint64_t stats[5]);
/* Device memory of the server's lanes: mem[0] the bytes their arenas hold now, mem[1]
 * what admission charges now (per lane the larger of its arenas and the estimate of the
 * batch it is compiling), mem[2] the largest charge seen after a compile, mem[3] the
 * budget.  A batch is admitted only when the charges fit in the budget: an idle lane
 * frees its arenas when a queued request needs the memory, and a lane whose arenas
 * outgrew its batch's estimate frees them after the compile, so mem[0] <= mem[3] between
 * compiles. */
ptl_status ptl_server_memory(ptl_server* server, uint64_t mem[4]);
/* Destroys the server after the compiles in flight; queued requests are dropped. */
void ptl_server_destroy(ptl_server* server);
/* The monotonic clock of the server's times, in ns. */
uint64_t ptl_clock_ns(void);

/* Kernel launches the library has issued so far (all generators of the process). */
uint64_t ptl_kernel_launches(void);

/* Library and device facts: CUDA runtime/driver versions, device name. */
ptl_status ptl_device_info(int device, char* name, size_t name_len, int* sm_count,
                           int* cc_major, int* cc_minor);

#ifdef __cplusplus
}
#endif

#endif
