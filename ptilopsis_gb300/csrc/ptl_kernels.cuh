// Kernel launch interface of the GB300 code generator (ptl_kernels.cu).
#pragma once

#include <cuda_runtime.h>

#include "ptl_device.h"
#include "ptl_stages.cuh"
#include "ptl_sort.cuh"
#include "ptl_scalar.cuh"

namespace ptl {

// Device scratch that a compile needs besides the Prog arrays; sized by the arena.
struct SortScratch {
    unsigned long long* a;     // (key, index) pairs, n
    uint32_t* apos;            // L-stop positions by rank, n
    uint32_t* bpos;            // R-stop positions by rank from the right, n
    SortSeg* seg[2];           // segment lists of this and the next round
    uint32_t seg_cap;
    uint32_t* tile_seg;        // tile -> segment
    uint32_t* tile_l;          // L-stop count per tile, then its exclusive offset
    uint32_t* tile_r;
    uint32_t* stops;           // per tile: its keys' L-stop bits, then their R-stop bits
                               // (kSortTile / 32 words each), written by the count pass
    uint32_t tile_cap;
    uint32_t* leaf;            // leaf ranges (first, last)
    uint32_t* heap;            // heap-sorted ranges
    uint32_t leaf_cap;
    uint32_t* local;           // ranges of at most kSortBlock keys (first, last, depth budget),
                               // finished one block each (k_sort_block)
    uint32_t* equal;           // equal-key ranges (first, last) found by the rounds
    uint32_t* counters;        // [0] tiles [1] next segments [2] leaves [3] heaps [4] segments of
                               // this round [5] capacity overflow [6] block ranges [7] equal ranges
};

constexpr size_t kScanTileElems = 4096;  // elements per scan tile (ptl_kernels.cu)

struct ScanScratch {
    unsigned long long* status;  // per tile: (flag << 32) | value
    uint32_t* counter;           // dynamic tile ticket
    uint32_t tile_cap;
};

// Kernel launches issued by this library since load (counted at each launch site).
uint64_t launch_count();
void note_launch();

// Element-wise stages (grid-stride launches of the per-thread functions).
void launch_ingest(const Prog& P, cudaStream_t s);  // input checks + copy; flags[3]: max_depth reached
void launch_preprocess(const Prog& P, cudaStream_t s);
void launch_count_scan(const Prog& P, const ScanScratch& sc, cudaStream_t s);
void launch_fix(const Prog& P, cudaStream_t s);
void launch_decl_scan(const Prog& P, uint32_t* flags_tmp, const ScanScratch& sc, cudaStream_t s);
void launch_functab(const Prog& P, uint32_t* meta, cudaStream_t s);

void launch_gen(const Prog& P, cudaStream_t s);
cudaError_t run_optimize(const Prog& P, cudaStream_t s, uint32_t* sweeps_out);
cudaError_t run_regalloc_steps(const Prog& P, cudaStream_t s, bool* serial_out, bool row0_hash);
// Lane-0 passes too wide for one block: programs with more than kRaClusterMin lane-0
// groups (at most 8,192) run theirs on a thread-block cluster when the device can place
// it.  ra_cluster_fits tells whether it can; launch_ra_wide launches the program's
// independent functions (Pfree: no definition positions), then the cluster pass (P0),
// and sets *launched, or launches nothing.
constexpr uint32_t kRaClusterMin = 1024;
bool ra_cluster_fits(uint32_t G0);
cudaError_t launch_ra_wide(const Prog& P0, const Prog& Pfree, uint32_t G0, cudaStream_t s, bool* launched);
void launch_regalloc_count_scan(const Prog& P, const ScanScratch& sc, cudaStream_t s);
void launch_regalloc_emit(const Prog& P, cudaStream_t s);
void launch_fixjumps_scan(const Prog& P, const ScanScratch& sc, cudaStream_t s);
void launch_fixjumps_emit(const Prog& P, cudaStream_t s);

// The scalar generator's stages where they differ (ptl_scalar.cuh).  Register
// allocation: the cross check (functions naming each other's words take the serial
// order), then one thread per function or the serial kernel (regs: F x 64, steps: F),
// each leaving the preserve masks; the count scan with the preserve words (extra: wb8
// counts); the scatter, the moved function table and the frame words (claim: W2 keys).
void launch_preprocess_scalar(const Prog& P, cudaStream_t s);
void launch_gen_scalar(const Prog& P, cudaStream_t s);
cudaError_t scalar_regalloc_cross(const Prog& P, cudaStream_t s, bool* cross);
void launch_scalar_ra_free(const Prog& P, unsigned long long* preserve, cudaStream_t s);
void launch_scalar_ra_serial(const Prog& P, int32_t* regs, SRaStep* steps, unsigned long long* preserve,
                             cudaStream_t s);
void launch_scalar_ra_count_scan(const Prog& P, const unsigned long long* preserve, uint32_t* extra,
                                 const ScanScratch& sc, cudaStream_t s);
void launch_scalar_ra_emit(const Prog& P, const unsigned long long* preserve, unsigned long long* claim,
                           cudaStream_t s);

// Two partition rounds as one CUDA graph.  Every launch of a round takes its arguments
// from the scratch layout (pointers, capacities) and reads its counts on the device, and
// the segment lists alternate, so a pair of rounds ends where it began and replays as one
// graph launch.  Captured on first use and again when the layout changes.
struct SortRoundGraph {
    cudaGraphExec_t exec = nullptr;
    SortScratch ss{};
    ErrorWord* err = nullptr;
    SortRoundGraph() = default;
    SortRoundGraph(const SortRoundGraph&) = delete;
    SortRoundGraph& operator=(const SortRoundGraph&) = delete;
    ~SortRoundGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// Depth-order emulation; returns a CUDA error and needs the host for its round loop.
cudaError_t run_depth_sort(const Prog& P, const SortScratch& ss, cudaStream_t s, uint32_t* rounds_out,
                           SortRoundGraph* graph = nullptr);

// Introsort rounds over prepared segments (ss.seg[0], counters), then heaps and leaves.
// With graph, rounds run as replays of a captured pair.
cudaError_t run_sort_rounds(const SortScratch& ss, uint32_t nseg0, uint32_t first_batch, uint32_t max_rounds,
                            ErrorWord* err, cudaStream_t s, uint32_t* rounds_out, SortRoundGraph* graph = nullptr);

// ---- batched programs: per-program Prog views in device memory (progs[B]); off[B+1]
// holds each program's first tile for the stage's element count.
struct BatchLaunch {
    const Prog* progs;
    const uint32_t* off;   // tile table built with `tile` elements per tile
    uint32_t B;
    cudaStream_t s;
    uint32_t tile;
};
enum class BatchStage {
    Ingest, Preprocess, Fix, Functab, Gen, OptMark, OptFinal, InitLifetime, Cross, RaHist, Spill,
    Scatter, RaFunctab, FjEmit, FjFunctab,
    // the scalar generator's (ptl_scalar.cuh): preprocess, isn_gen, preserve counts
    // (per function), scatter (per word), the function table after regalloc (per
    // function), the frame words and preserve stores (3 items per function)
    PreprocessScalar, GenScalar, SPreserveCounts, SScatter, SFunctab, SFrames
};
enum class BatchScan { Count, Decl, RaCount, FjSize, SRaCount };
uint32_t batch_tile();       // default elements per tile of the element-wise stages
// Tile sizes the element-wise kernels and the optimize sweeps accept (powers of two).
bool batch_tile_ok(uint32_t tile);
bool batch_sweep_tile_ok(uint32_t tile);
uint32_t batch_scan_tile();  // elements per scan tile
void batch_stage(BatchStage st, const BatchLaunch& bl, uint32_t total, uint32_t* meta);

// Batched arenas: a program's region in an array family holds kArenaFront zero elements,
// its elements, then zeros up to the next multiple of 32 that is at least kArenaBack past
// them (stages read a little before and past a program's elements).
constexpr uint64_t kArenaFront = 16, kArenaBack = 80;
PTL_HD uint64_t arena_region(uint64_t count) { return (count + kArenaFront + kArenaBack + 31) & ~uint64_t(31); }
// Families whose elements the stages write in full before reading them; only the pads
// need zeroing, which batch_guards does (per program, region(count) - written elements):
//   Nodes: nt rt nd1 nd par ci dep loc0 loc fflag, written [0, nb8), count nb8;
//   Words: used_instrs spill roffs, written from [0, W), count wb8;
//   Words2: joffs, written [0, w2b8), count w2b8 + 16.
enum class ArenaGuard { Nodes, Words, Words2 };
void batch_guards(ArenaGuard g, const BatchLaunch& bl, uint32_t total);
void batch_sort_keys(const BatchLaunch& bl, uint32_t total, unsigned long long* a, const uint64_t* aoff, bool out);
// One optimize sweep over the tiles marked in cur (all when cur is null); marks in next
// the tiles a cleared mark makes live again.  Both hold total + 1 bytes: the last says
// whether any tile is marked (a sweep with none returns at once).  Valid only when the
// OptMark stage found every virtual result to be its instruction's own word (its flag
// 0); otherwise pass cur = null.
void batch_sweep(const BatchLaunch& bl, uint32_t total, uint32_t* changed, const uint8_t* cur, uint8_t* next);

// One input field of every program copied from the caller's host arrays into the device
// input arena by a kernel that reads host memory directly (devices with coherent access
// to pageable memory).  Program p's elements go to dst + din[p] * esize, din[p] a multiple
// of 16; the table bl.off counts tiles of kGatherTile elements per program.
struct HostGather {
    const void* const* src;  // [B] host arrays of this field
    const uint64_t* din;     // [B] first element in dst
    const uint64_t* n;       // [B] elements
    uint8_t* dst;
    uint32_t esize;          // 1 or 4
};
constexpr uint32_t kGatherTile = 32768;
void batch_gather_host(const BatchLaunch& bl, uint32_t total, const HostGather& g);
// A kernel copying bytes (a multiple of 16, both 16-byte aligned) from host memory it
// reads directly into device memory.
cudaError_t read_host(const void* src, void* dst, size_t bytes, cudaStream_t s);
// Copies bytes between memories a kernel can address (device memory, pinned host memory,
// pageable host memory where the device accesses it coherently), both 16-byte aligned,
// with kernel loads and stores: over the host link faster than the copy engine here.
cudaError_t kernel_copy(const void* src, void* dst, size_t bytes, cudaStream_t s);
void batch_scan(BatchScan which, const BatchLaunch& bl, uint32_t tiles, const ScanScratch& sc, uint32_t* meta);
void batch_sizes(bool w3, const Prog* progs, const uint32_t* list, uint32_t count, uint32_t* meta, cudaStream_t s);
// ra_order of each listed program: its independent functions, longest first.
void batch_free_order(const Prog* progs, const uint32_t* list, uint32_t count, cudaStream_t s);
void batch_serial(const Prog* progs, const uint32_t* list, uint32_t count, cudaStream_t s);
// Register allocation steps of n programs in one persistent launch: program order[k]
// owns work items item_off[k] .. item_off[k+1] (its independent functions in tiles of
// batch_ra_threads(max_g0), then its lane-0 pass, which follows their progress through
// the program's ra_chunks record: histogram (BatchStage::RaHist) then zeroed counts).
uint32_t batch_ra_threads(uint32_t max_g0);
// The scalar generator's register allocation of the listed programs' functions, one warp
// per function (a tile: scalar_warp_fns() functions of one program; the tile table over
// F in bl), each warp with `stride` symbol bytes (at least the listed programs' longest
// function, at most scalar_warp_cap()).  The serial and tile forms run per program
// through launch_scalar_ra_serial / launch_scalar_ra_free.
void batch_scalar_ra_warp(const BatchLaunch& bl, uint32_t total, uint32_t stride);
uint32_t scalar_warp_fns();
uint32_t scalar_warp_cap();
// share: the part of the device's resident blocks the persistent launch may take (1 =
// all; less leaves room for other streams' kernels, e.g. a compile server's other lanes).
cudaError_t batch_regalloc(const Prog* progs, const uint32_t* item_off, const uint32_t* order, uint32_t n,
                           uint32_t items, uint32_t max_g0, uint32_t* queue, cudaStream_t s, double share = 1.0);

}  // namespace ptl
