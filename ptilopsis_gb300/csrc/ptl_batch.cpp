// Batched compilation and the compile server (include/ptl_codegen.h: ptl_batch_*,
// ptl_server_*).
//
// Neither has a counterpart in the reference, which compiles one tree per process
// (src/main.cpp:121-157).  A batch runs all its programs through the batched pipeline
// (one launch per stage step for the whole batch).  The server keeps a pool of worker
// threads, each owning one generator: its device arena stays resident and grows to the
// largest program it has compiled, and its stream lets the compiles of different workers
// overlap on the GPU.  The server batches queued requests through batched pipelines.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/ptl_codegen.h"
#include "ptl_bpipe.h"

namespace {

uint64_t now_ns() {
    return static_cast<uint64_t>(
        std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
            .count());
}

// One compiled program, copied out of the pipeline that made it.
struct Result {
    ptl_status status = PTL_OK;
    std::string error;  // detail of a batch-wide failure
    std::vector<uint32_t> words, starts, ends, sizes, ids;
};

// Device footprint of a batch of n nodes in all, for admission: the pipeline's arrays
// (about 210 bytes per node with the word arrays at ~1.25 words per node and the sort and
// regalloc scratch), the arenas' 25% growth margin, and fixed scratch.  A lane that
// finds its arenas past the estimate after a compile frees them (see ptl_server::run),
// so the budget holds between compiles whatever the estimate.
uint64_t footprint(size_t n) { return 64ull * 1024 * 1024 + 288ull * n; }

}  // namespace

// ===================================================================== batch
// One batched pipeline (ptl_bpipe.cu): every stage step is one launch for all programs.
struct ptl_batch {
    std::unique_ptr<ptl::BatchPipeline> pipe;
    std::vector<ptl::BatchResult> results;
    uint64_t last_ns = 0;
};

extern "C" ptl_status ptl_batch_create(int device, int workers, ptl_batch** out) {
    if (!out || workers < 1 || workers > 256) return PTL_BAD_ARGUMENT;
    ptl_batch* b = new (std::nothrow) ptl_batch;
    if (!b) return PTL_OOM;
    ptl_status st = PTL_OK;
    b->pipe.reset(ptl::BatchPipeline::create(device, workers, &st));
    if (!b->pipe) {
        delete b;
        return st;
    }
    *out = b;
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_compile(ptl_batch* b, const ptl_ast_view* trees, size_t count) {
    if (!b || (!trees && count)) return PTL_BAD_ARGUMENT;
    const uint64_t t0 = now_ns();
    const ptl_status st = b->pipe->compile(trees, count, b->results);
    b->last_ns = now_ns() - t0;
    if (st != PTL_OK) return st;
    for (const ptl::BatchResult& r : b->results)
        if (r.status != PTL_OK) return r.status;
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_status(const ptl_batch* b, size_t k) {
    if (!b || k >= b->results.size()) return PTL_BAD_ARGUMENT;
    return b->results[k].status;
}

extern "C" ptl_status ptl_batch_words(const ptl_batch* b, size_t k, const uint32_t** words, size_t* count) {
    if (!b || !words || !count || k >= b->results.size()) return PTL_BAD_ARGUMENT;
    const ptl::BatchResult& r = b->results[k];
    if (r.status != PTL_OK) return r.status;
    *words = r.words;
    *count = r.count;
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_function_table(const ptl_batch* b, size_t k, const uint32_t** starts,
                                               const uint32_t** ends, const uint32_t** sizes, const uint32_t** ids,
                                               size_t* count) {
    if (!b || !starts || !ends || !sizes || !ids || !count || k >= b->results.size()) return PTL_BAD_ARGUMENT;
    const ptl::BatchResult& r = b->results[k];
    if (r.status != PTL_OK) return r.status;
    *starts = r.starts;
    *ends = r.ends;
    *sizes = r.sizes;
    *ids = r.ids;
    *count = r.functions;
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_sizes(const ptl_batch* b, size_t k, uint64_t sizes[4]) {
    if (!b || !sizes || k >= b->results.size()) return PTL_BAD_ARGUMENT;
    const ptl::BatchResult& r = b->results[k];
    if (r.status != PTL_OK) return r.status;
    sizes[0] = r.nodes;
    sizes[1] = r.words_gen;
    sizes[2] = r.words_ra;
    sizes[3] = r.count;
    return PTL_OK;
}

extern "C" uint64_t ptl_batch_elapsed_ns(const ptl_batch* b) { return b ? b->last_ns : 0; }

extern "C" ptl_status ptl_batch_stage_ns(const ptl_batch* b, uint64_t ns[7]) {
    if (!b || !ns) return PTL_BAD_ARGUMENT;
    b->pipe->stage_ns(ns);
    return PTL_OK;
}

extern "C" uint64_t ptl_batch_device_ns(const ptl_batch* b) { return b ? b->pipe->device_ns() : 0; }
extern "C" uint64_t ptl_batch_depth_sort_ns(const ptl_batch* b) { return b ? b->pipe->depth_sort_ns() : 0; }

extern "C" ptl_status ptl_batch_copied_bytes(const ptl_batch* b, uint64_t* h2d, uint64_t* d2h) {
    if (!b) return PTL_BAD_ARGUMENT;
    b->pipe->copied_bytes(h2d, d2h);
    return PTL_OK;
}

extern "C" const char* ptl_batch_last_error(const ptl_batch* b) { return b ? b->pipe->last_error() : ""; }

extern "C" ptl_status ptl_batch_host_ns(const ptl_batch* b, uint64_t ns[3]) {
    if (!b || !ns) return PTL_BAD_ARGUMENT;
    b->pipe->host_ns(ns);
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_set_tiles(ptl_batch* b, uint32_t elem_tile, uint32_t sweep_tile) {
    if (!b) return PTL_BAD_ARGUMENT;
    return b->pipe->set_tiles(elem_tile, sweep_tile) ? PTL_OK : PTL_BAD_ARGUMENT;
}

extern "C" ptl_status ptl_batch_set_regalloc_share(ptl_batch* b, double share) {
    if (!b || !(share > 0.0 && share <= 1.0)) return PTL_BAD_ARGUMENT;
    b->pipe->set_regalloc_share(share);
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_set_scalar(ptl_batch* b, int scalar) {
    if (!b) return PTL_BAD_ARGUMENT;
    b->pipe->set_scalar(scalar != 0);
    return PTL_OK;
}

extern "C" ptl_status ptl_batch_tiles(const ptl_batch* b, uint32_t tiles[2]) {
    if (!b || !tiles) return PTL_BAD_ARGUMENT;
    b->pipe->tiles(tiles);
    return PTL_OK;
}

extern "C" void ptl_batch_destroy(ptl_batch* b) { delete b; }

// ===================================================================== server
namespace {

// A request owns a copy of its tree (the caller's arrays may go away after submit), or,
// submitted with PTL_SUBMIT_BORROW, refers to the caller's arrays until it is released.
struct Request {
    uint64_t ticket = 0;
    size_t n = 0, max_depth = 0;
    std::vector<uint8_t> type, rtype;
    std::vector<int32_t> parent, depth, child;
    std::vector<uint32_t> data;
    bool borrowed = false;
    bool scalar = false;  // the scalar generator's semantics (PTL_SUBMIT_SCALAR)
    ptl_ast_view borrowed_view{};
    uint64_t bytes = 0;        // admission estimate
    uint64_t t_submit = 0, t_start = 0, t_done = 0;
    bool done = false;
    Result result;

    ptl_ast_view view() const {
        if (borrowed) return borrowed_view;
        return ptl_ast_view{n,           max_depth,    type.data(),  rtype.data(), parent.data(),
                            depth.data(), child.data(), data.data(), 0};
    }
};

}  // namespace

struct ptl_server {
    int device = 0;
    uint64_t budget = 0;
    uint64_t in_use = 0;       // admission estimates of the compiles in flight
    // Device memory per lane: what its arenas hold (resident, measured after each compile)
    // and the estimate of the batch it is compiling (reserved, 0 when idle).  A lane is
    // charged the larger of the two, and a batch is admitted only when every lane's charge
    // fits in the budget; an idle lane whose resident arenas stand in the way of a queued
    // request is asked to free them (trim).
    std::vector<uint64_t> resident, reserved;
    std::vector<uint8_t> trim;
    uint64_t charged(size_t skip = SIZE_MAX) const {
        uint64_t t = 0;
        for (size_t w = 0; w < resident.size(); ++w)
            if (w != skip) t += std::max(resident[w], reserved[w]);
        return t;
    }
    uint64_t max_batch_nodes = 64ull << 20;
    static constexpr size_t kCopyThreads = 6;                 // result copies of one batch
    static constexpr uint64_t kCopyWordsPerThread = 4u << 20;  // (16 MB of words a thread at least)
    static constexpr size_t kLookAhead = 4096;  // queued requests examined per batch formed
    // Requests below small_nodes are "small"; lanes w < small_lanes take only those, so a
    // small request never waits behind a large one whose register allocation chain sets a
    // batch's duration.  The other lanes prefer large requests and take small ones when no
    // large request is queued.
    uint64_t small_nodes = 64ull << 10;
    size_t small_lanes = 1;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    // queued requests by size class (0: small, 1: large), each in arrival order, for the
    // AVX generator's semantics (mode 0) and the scalar generator's (mode 1); a lane takes
    // from the front, so a batch leaves its queue in O(1) per request however long the
    // queue has grown
    std::deque<std::shared_ptr<Request>> queue[2][2];
    // The mode whose queue of class c has the earliest request at its front.
    int mode_for(int c) const {
        if (queue[1][c].empty()) return 0;
        if (queue[0][c].empty()) return 1;
        return queue[1][c].front()->t_submit < queue[0][c].front()->t_submit ? 1 : 0;
    }
    std::unordered_map<uint64_t, std::shared_ptr<Request>> all;
    std::vector<std::thread> lanes;
    std::vector<std::unique_ptr<ptl::BatchPipeline>> pipes;
    uint64_t next_ticket = 1;
    bool stopping = false;
    uint64_t completed = 0, nodes_done = 0, batches = 0;
    uint64_t peak_resident = 0;  // largest total of the lanes' charges seen after a compile

    // Continuous batching: a free lane takes every queued request of its size class, in
    // arrival order, that fits the memory left in the budget and the batch cap (a later
    // request that fits may pass one that does not) -- a large-request lane takes small
    // requests when it has no large one -- and compiles them through its batched pipeline
    // while the other lanes keep taking the requests that arrive meanwhile.
    void run(size_t w) {
        std::vector<std::shared_ptr<Request>> batch;
        bool batch_scalar = false;
        std::vector<ptl_ast_view> views;
        std::vector<ptl::BatchResult> res;
        const bool prefer_small = w < small_lanes;
        for (;;) {
            batch.clear();
            {
                std::unique_lock<std::mutex> lk(mu);
                for (;;) {
                    if (stopping) return;
                    if (trim[w]) {  // another lane needs the memory this idle lane's arenas hold
                        lk.unlock();  // cudaFree waits for the device: not under the lock
                        pipes[w]->release_memory();
                        lk.lock();
                        resident[w] = 0;
                        trim[w] = 0;
                        cv_work.notify_all();
                        continue;
                    }
                    const uint64_t others = charged(w);
                    uint64_t need_min = UINT64_MAX;  // smallest estimate of a request that waits for memory
                    uint64_t batch_bytes = 0;
                    for (int pass = 0; pass < (prefer_small ? 1 : 2) && batch.empty(); ++pass) {
                        const bool want_small = (pass == 0) == prefer_small;
                        uint64_t nodes = 0;
                        const int c = want_small ? 0 : 1;
                        batch_scalar = mode_for(c) == 1;
                        std::deque<std::shared_ptr<Request>>& q = queue[batch_scalar ? 1 : 0][c];
                        // a request that does not fit may be passed by later ones that do, within a
                        // bounded look-ahead (the lock is held while a batch is formed)
                        size_t looked = 0;
                        for (auto it = q.begin(); it != q.end() && nodes < max_batch_nodes && looked < kLookAhead;
                             ++looked) {
                            const std::shared_ptr<Request>& r = *it;
                            const uint64_t need = footprint(nodes + r->n);
                            const bool fits = others + std::max(resident[w], need) <= budget &&
                                              (batch.empty() || nodes + r->n <= max_batch_nodes);
                            if (fits) {
                                nodes += r->n;
                                batch.push_back(r);
                                it = q.erase(it);  // at the front unless an earlier request waits
                            } else {
                                if (batch.empty()) need_min = std::min(need_min, need);
                                ++it;
                            }
                        }
                        batch_bytes = footprint(nodes);
                    }
                    if (!batch.empty()) {
                        reserved[w] = batch_bytes;
                        for (auto& r : batch) in_use += r->bytes;
                        break;
                    }
                    if (need_min != UINT64_MAX) {  // a request waits for memory
                        if (resident[w] > 0 && others + need_min <= budget) {
                            // this lane's own high-water arenas are what stands in the way
                            lk.unlock();
                            pipes[w]->release_memory();
                            lk.lock();
                            resident[w] = 0;
                            continue;
                        }
                        bool asked = false;  // else the idle lanes' arenas
                        for (size_t v = 0; v < pipes.size(); ++v) {
                            if (v != w && reserved[v] == 0 && resident[v] > 0 && !trim[v]) {
                                trim[v] = 1;
                                asked = true;
                            }
                        }
                        if (asked) cv_work.notify_all();
                    }
                    cv_work.wait(lk);
                }
            }
            const uint64_t t0 = now_ns();
            views.clear();
            for (auto& r : batch) {
                r->t_start = t0;
                views.push_back(r->view());
            }
            pipes[w]->set_scalar(batch_scalar);
            const ptl_status st = pipes[w]->compile(views.data(), views.size(), res);
            uint64_t held = pipes[w]->device_bytes();
            // The results leave the pipeline's output buffers before the lane's next compile
            // overwrites them; a large batch's (hundreds of MB) on several threads, since
            // the lane takes no new batch meanwhile.
            auto copy_out = [&](size_t k) {
                Result& out = batch[k]->result;
                if (st != PTL_OK) {
                    out.status = st;
                    const char* why = pipes[w]->last_error();
                    out.error = why ? why : "";
                    return;
                }
                const ptl::BatchResult& r = res[k];
                out.status = r.status;
                if (r.status != PTL_OK) return;
                out.words.assign(r.words, r.words + r.count);
                out.starts.assign(r.starts, r.starts + r.functions);
                out.ends.assign(r.ends, r.ends + r.functions);
                out.sizes.assign(r.sizes, r.sizes + r.functions);
                out.ids.assign(r.ids, r.ids + r.functions);
            };
            uint64_t words = 0;
            if (st == PTL_OK)
                for (size_t k = 0; k < batch.size(); ++k) words += res[k].status == PTL_OK ? res[k].count : 0;
            const size_t helpers = std::min<size_t>({kCopyThreads - 1, batch.size() - 1, words / kCopyWordsPerThread});
            if (helpers == 0) {
                for (size_t k = 0; k < batch.size(); ++k) copy_out(k);
            } else {
                std::atomic<size_t> next{0};
                auto drain = [&] {
                    for (size_t k = next.fetch_add(1); k < batch.size(); k = next.fetch_add(1)) copy_out(k);
                };
                std::vector<std::thread> th;
                for (size_t h = 0; h < helpers; ++h) th.emplace_back(drain);
                drain();
                for (auto& t : th) t.join();
            }
            bool give_back = false;
            {
                std::lock_guard<std::mutex> lk(mu);
                const uint64_t t1 = now_ns();
                for (auto& r : batch) {
                    r->t_done = t1;
                    r->done = true;
                    in_use -= r->bytes;
                    ++completed;
                    nodes_done += r->n;
                }
                ++batches;
                // the arenas stay charged until they are freed
                resident[w] = held;
                reserved[w] = 0;
                peak_resident = std::max(peak_resident, charged());
                give_back = charged() > budget;  // they outgrew the batch's estimate
            }
            if (give_back) {
                pipes[w]->release_memory();
                std::lock_guard<std::mutex> lk(mu);
                resident[w] = 0;
            }
            cv_done.notify_all();
            cv_work.notify_all();
        }
    }
};

extern "C" ptl_status ptl_server_create(int device, int slots, uint64_t memory_budget, ptl_server** out) {
    if (!out || slots < 1 || slots > 16 || memory_budget == 0) return PTL_BAD_ARGUMENT;
    ptl_server* s = new (std::nothrow) ptl_server;
    if (!s) return PTL_OOM;
    s->device = device;
    s->budget = memory_budget;
    s->small_lanes = slots > 1 ? static_cast<size_t>(slots) / 2 : 0;  // one lane takes everything
    s->resident.assign(static_cast<size_t>(slots), 0);
    s->reserved.assign(static_cast<size_t>(slots), 0);
    s->trim.assign(static_cast<size_t>(slots), 0);
    for (int w = 0; w < slots; ++w) {
        ptl_status st = PTL_OK;
        // small-request lanes run at the highest stream priority: their short, latency-bound
        // batches get SMs ahead of the large batches' blocks
        s->pipes.emplace_back(ptl::BatchPipeline::create(device, 8, &st, static_cast<size_t>(w) < s->small_lanes));
        // a large-request lane's persistent regalloc launch leaves half the SMs' block slots
        // to the small-request lanes
        if (s->pipes.back() && s->small_lanes > 0 && static_cast<size_t>(w) >= s->small_lanes)
            s->pipes.back()->set_regalloc_share(0.5);
        if (!s->pipes.back()) {
            s->pipes.clear();
            delete s;
            return st;
        }
    }
    for (int w = 0; w < slots; ++w) s->lanes.emplace_back([s, w] { s->run(static_cast<size_t>(w)); });
    *out = s;
    return PTL_OK;
}

extern "C" ptl_status ptl_server_submit(ptl_server* s, const ptl_ast_view* tree, uint64_t* ticket) {
    return ptl_server_submit_flags(s, tree, 0, ticket);
}

extern "C" ptl_status ptl_server_submit_flags(ptl_server* s, const ptl_ast_view* tree, uint32_t flags,
                                              uint64_t* ticket) {
    if (!s || !tree || !ticket || tree->on_device || (flags & ~(PTL_SUBMIT_BORROW | PTL_SUBMIT_SCALAR)))
        return PTL_BAD_ARGUMENT;
    auto req = std::make_shared<Request>();
    const size_t n = tree->n;
    req->n = n;
    req->max_depth = tree->max_depth;
    req->bytes = footprint(n);
    req->scalar = (flags & PTL_SUBMIT_SCALAR) != 0;
    if (req->bytes > s->budget) return PTL_ADMISSION_DENIED;  // could never be admitted
    if (n && (!tree->type || !tree->rtype || !tree->parent || !tree->depth || !tree->child_idx || !tree->data))
        return PTL_BAD_ARGUMENT;
    if (flags & PTL_SUBMIT_BORROW) {
        req->borrowed = true;
        req->borrowed_view = *tree;
    } else {
        req->type.assign(tree->type, tree->type + n);
        req->rtype.assign(tree->rtype, tree->rtype + n);
        req->parent.assign(tree->parent, tree->parent + n);
        req->depth.assign(tree->depth, tree->depth + n);
        req->child.assign(tree->child_idx, tree->child_idx + n);
        req->data.assign(tree->data, tree->data + n);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        req->ticket = s->next_ticket++;
        req->t_submit = now_ns();
        s->all[req->ticket] = req;
        s->queue[req->scalar ? 1 : 0][n < s->small_nodes ? 0 : 1].push_back(req);
        *ticket = req->ticket;
    }
    s->cv_work.notify_one();
    return PTL_OK;
}

// Waits (wait != 0) or checks whether the ticket is done; *done receives the state.
extern "C" ptl_status ptl_server_poll(ptl_server* s, uint64_t ticket, int wait, int* done) {
    if (!s || !done) return PTL_BAD_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) return PTL_BAD_ARGUMENT;
    std::shared_ptr<Request> req = it->second;
    if (wait) s->cv_done.wait(lk, [&] { return req->done; });
    *done = req->done ? 1 : 0;
    return req->done ? req->result.status : PTL_OK;
}

extern "C" ptl_status ptl_server_result(ptl_server* s, uint64_t ticket, const uint32_t** words, size_t* count,
                                        const uint32_t** starts, const uint32_t** ends, const uint32_t** sizes,
                                        const uint32_t** ids, size_t* functions) {
    if (!s || !words || !count) return PTL_BAD_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end() || !it->second->done) return PTL_BAD_ARGUMENT;
    const Result& r = it->second->result;
    if (r.status != PTL_OK) return r.status;
    *words = r.words.data();
    *count = r.words.size();
    if (starts && ends && sizes && ids && functions) {
        *starts = r.starts.data();
        *ends = r.ends.data();
        *sizes = r.sizes.data();
        *ids = r.ids.data();
        *functions = r.starts.size();
    }
    return PTL_OK;
}

// Detail of a finished ticket's batch-wide failure ("" when there was none).
extern "C" const char* ptl_server_error(ptl_server* s, uint64_t ticket) {
    if (!s) return "";
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end() || !it->second->done) return "";
    return it->second->result.error.c_str();
}

// Submit, start and completion times (steady clock, ns) of a finished ticket.
extern "C" ptl_status ptl_server_times(ptl_server* s, uint64_t ticket, uint64_t times[3]) {
    if (!s || !times) return PTL_BAD_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end() || !it->second->done) return PTL_BAD_ARGUMENT;
    times[0] = it->second->t_submit;
    times[1] = it->second->t_start;
    times[2] = it->second->t_done;
    return PTL_OK;
}

extern "C" ptl_status ptl_server_release(ptl_server* s, uint64_t ticket) {
    if (!s) return PTL_BAD_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end() || !it->second->done) return PTL_BAD_ARGUMENT;
    s->all.erase(it);
    return PTL_OK;
}

// stats: completed, nodes compiled, queued, in flight (admission bytes), batches run
extern "C" ptl_status ptl_server_stats(ptl_server* s, uint64_t stats[5]) {
    if (!s || !stats) return PTL_BAD_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    stats[0] = s->completed;
    stats[1] = s->nodes_done;
    stats[2] = s->queue[0][0].size() + s->queue[0][1].size() + s->queue[1][0].size() + s->queue[1][1].size();
    stats[3] = s->in_use;
    stats[4] = s->batches;
    return PTL_OK;
}

extern "C" ptl_status ptl_server_memory(ptl_server* s, uint64_t mem[4]) {
    if (!s || !mem) return PTL_BAD_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    uint64_t held = 0;
    for (uint64_t r : s->resident) held += r;
    mem[0] = held;
    mem[1] = s->charged();
    mem[2] = s->peak_resident;
    mem[3] = s->budget;
    return PTL_OK;
}

extern "C" uint64_t ptl_clock_ns(void) { return now_ns(); }

extern "C" void ptl_server_destroy(ptl_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopping = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->lanes) t.join();
    delete s;
}
