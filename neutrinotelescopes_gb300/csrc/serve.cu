// serve.cu -- continuous-batching event server (include/ntp.h, ntp_server_*).
//
// The reference simulates one event per propagate_photons call
// (photon_prop_cuda.jl:804-817), each launch allocating its own hit buffer.
// Here events arrive as requests; the server keeps a FIFO queue, admits events
// while their hit reservations fit into a device-resident arena (the HBM
// budget), packs the admitted events into one persistent propagation launch
// and keeps their hits in the arena until the caller releases them.
//
// Each of two batch slots owns a stream, pinned input / output blocks and a
// CUDA graph captured once: H2D copy of the batch tables, a set-up kernel that
// installs the arena ranges of newly placed events (and zeroes their hit
// counters), the propagation kernel, a kernel gathering the batch's event
// hit counts, D2H copy of those counts.  A launch rewrites the pinned input
// block, updates the propagation node's parameters and replays the graph.
// With two slots a new batch is queued while the previous one runs, so its
// blocks take over SMs as the previous launch drains.
//
// Photon k of event e draws from Philox counter (draw, k, e): an event's hits
// are the same whatever batch it runs in, and whether it runs whole or in
// chunks (a chunk [a, b) passes a as its photon offset).  Every placed event
// owns an output slot (device hit counter, arena base and reservation); its
// chunks write to it.  An event has at most one chunk in flight, so the
// count gathered after its last chunk is final; a count above the
// reservation is exact, and the event goes back to the head of the queue
// with the exact reservation and runs again from its first photon.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "ntp_internal.h"

namespace {

// First-fit allocator of hit records over [0, size), coalescing on release.
class Arena {
  public:
    explicit Arena(uint64_t size = 0) : size_(size) {
        if (size) free_[0] = size;
    }
    bool alloc(uint64_t n, uint64_t* off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const uint64_t rest = it->second - n, start = it->first + n;
            free_.erase(it);
            if (rest) free_[start] = rest;
            used_ += n;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t n) {
        if (!n) return;
        used_ -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t size() const { return size_; }
    uint64_t used() const { return used_; }

  private:
    std::map<uint64_t, uint64_t> free_;
    uint64_t size_ = 0, used_ = 0;
};

enum class State { Queued, Running, Done };

struct Event {
    uint32_t id = 0;
    ntp_source src{};
    State state = State::Queued;
    uint64_t reserve = 0, offset = 0, n_hits = 0;
    uint64_t launched = 0;  // photons handed to batches so far
    bool placed = false;
    bool in_flight = false;
    int out = -1;           // output slot (device counter, base, cap) while placed
    int reruns = 0, batch_events = 0;
    double t_submit = 0, t_launch = 0, t_done = 0;
};

constexpr int kOutSlots = 65536;  // events placed at one time

// Installs the arena ranges of the events placed for this batch: header
// word 1 = their number, then (slot, base, cap) triples.
__global__ void serve_setup_kernel(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ slot,
                                   const unsigned long long* __restrict__ base,
                                   const unsigned long long* __restrict__ cap, unsigned long long* __restrict__ count,
                                   unsigned long long* __restrict__ ev_base, unsigned long long* __restrict__ ev_cap) {
    const uint32_t n = hdr[1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t o = slot[i];
        if (o >= static_cast<uint32_t>(kOutSlots)) continue;
        ev_base[o] = base[i];
        ev_cap[o] = cap[i];
        count[o] = 0;
    }
}

// The hit counts of the batch's entries (header word 0 = their number).
__global__ void serve_gather_kernel(const uint32_t* __restrict__ hdr, const uint32_t* __restrict__ out_slot,
                                    const unsigned long long* __restrict__ count, unsigned long long* __restrict__ dst) {
    const uint32_t n = hdr[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t o = out_slot[i];
        dst[i] = o < static_cast<uint32_t>(kOutSlots) ? count[o] : 0ull;
    }
}

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t kernel_node = nullptr;
    unsigned char* d_in = nullptr;
    unsigned char* h_in = nullptr;
    unsigned char* d_out = nullptr;
    unsigned char* h_out = nullptr;
    std::vector<uint32_t> events;
    bool busy = false;
};

size_t align8(size_t x) { return (x + 7) / 8 * 8; }

}  // namespace

struct ntp_server {
    ntp_ctx* ctx = nullptr;
    ntp_server_config cfg{};
    ntp::PropParams world{};
    int grid = 0;
    size_t smem = 0;
    int n_max = 0;
    // byte offsets inside a slot's input / output blocks
    size_t off_hdr = 0, off_src = 0, off_prefix = 0, off_stream = 0, off_poff = 0, off_out = 0;
    size_t off_nslot = 0, off_nbase = 0, off_ncap = 0, in_bytes = 0;
    size_t off_count = 0, off_counters = 0, out_bytes = 0;
    ntp_hit* d_arena = nullptr;
    Arena arena;
    // output slots: device hit counters, arena bases and reservations
    unsigned long long* d_ev = nullptr;  // count[kOutSlots] | base[kOutSlots] | cap[kOutSlots]
    std::vector<int> free_out;
    std::deque<uint32_t> queue;
    std::unordered_map<uint32_t, Event> events;
    Slot slots[2];
    std::deque<ntp_event_result> ready;
    std::chrono::steady_clock::time_point t0;
    uint64_t n_batches = 0, n_photons = 0, n_completed = 0, n_released = 0;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

bool fail_cuda(ntp_server* s, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return false;
    std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
    ntp::set_ctx_error(s->ctx, msg.c_str());
    return true;
}

template <typename T>
T* at(unsigned char* base, size_t off) {
    return reinterpret_cast<T*>(base + off);
}

void fill_slot_params(const ntp_server* s, const Slot& sl, ntp::PropParams& p) {
    p = s->world;
    p.sources = at<const ntp_source>(sl.d_in, s->off_src);
    p.prefix = at<const unsigned long long>(sl.d_in, s->off_prefix);
    p.src_stream = at<const uint32_t>(sl.d_in, s->off_stream);
    p.src_photon_offset = at<const unsigned long long>(sl.d_in, s->off_poff);
    p.src_out = at<const uint32_t>(sl.d_in, s->off_out);
    p.src_hit_count = s->d_ev;
    p.src_hit_base = s->d_ev + kOutSlots;
    p.src_hit_cap = s->d_ev + 2 * kOutSlots;
    p.counters = at<unsigned long long>(sl.d_out, s->off_counters);
    p.hits = s->d_arena;
    p.capacity = s->arena.size();
}

// Captures the slot's graph: inputs H2D, counters zeroed, newly placed
// events installed, propagation, the batch's counts gathered and copied D2H.
bool capture_slot(ntp_server* s, Slot& sl) {
    ntp::PropParams p;
    fill_slot_params(s, sl, p);
    p.n_src = 1;
    p.total = 0;  // replaced at every launch
    p.chunk = 32;
    const uint32_t* hdr = at<const uint32_t>(sl.d_in, s->off_hdr);
    if (fail_cuda(s, cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture"))
        return false;
    cudaMemcpyAsync(sl.d_in, sl.h_in, s->in_bytes, cudaMemcpyHostToDevice, sl.stream);
    cudaMemsetAsync(sl.d_out, 0, s->out_bytes, sl.stream);
    serve_setup_kernel<<<64, 256, 0, sl.stream>>>(hdr, at<const uint32_t>(sl.d_in, s->off_nslot),
                                                  at<const unsigned long long>(sl.d_in, s->off_nbase),
                                                  at<const unsigned long long>(sl.d_in, s->off_ncap), s->d_ev,
                                                  s->d_ev + kOutSlots, s->d_ev + 2 * kOutSlots);
    ntp::launch_propagate(p, s->grid, sl.stream);
    serve_gather_kernel<<<64, 256, 0, sl.stream>>>(hdr, at<const uint32_t>(sl.d_in, s->off_out), s->d_ev,
                                                   at<unsigned long long>(sl.d_out, s->off_count));
    cudaMemcpyAsync(sl.h_out, sl.d_out, s->out_bytes, cudaMemcpyDeviceToHost, sl.stream);
    if (fail_cuda(s, cudaStreamEndCapture(sl.stream, &sl.graph), "cudaStreamEndCapture")) return false;
    if (fail_cuda(s, cudaGraphInstantiate(&sl.exec, sl.graph, 0), "cudaGraphInstantiate")) return false;
    size_t n = 0;
    if (fail_cuda(s, cudaGraphGetNodes(sl.graph, nullptr, &n), "cudaGraphGetNodes")) return false;
    std::vector<cudaGraphNode_t> nodes(n);
    if (fail_cuda(s, cudaGraphGetNodes(sl.graph, nodes.data(), &n), "cudaGraphGetNodes")) return false;
    // the propagation node: by its function, else by its launch shape (the
    // set-up and gather kernels run 64 blocks, the propagation one per SM slot)
    cudaGraphNode_t by_shape = nullptr;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        cudaGraphNodeGetType(nd, &t);
        if (t != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp{};
        if (cudaGraphKernelNodeGetParams(nd, &kp) != cudaSuccess) continue;
        if (kp.func == ntp::propagate_kernel_fn()) sl.kernel_node = nd;
        if (static_cast<int>(kp.gridDim.x) == s->grid && kp.sharedMemBytes == s->smem) by_shape = nd;
    }
    if (!sl.kernel_node) sl.kernel_node = by_shape;
    if (!sl.kernel_node) {
        ntp::set_ctx_error(s->ctx, "ntp_server: captured graph has no kernel node");
        return false;
    }
    return true;
}

void finish_event(ntp_server* s, Event& e, int status) {
    e.state = State::Done;
    e.t_done = s->now();
    if (e.out >= 0) {  // no kernel writes to the slot any more
        s->free_out.push_back(e.out);
        e.out = -1;
    }
    ntp_event_result r{};
    r.event_id = e.id;
    r.status = status;
    r.n_hits = e.n_hits;
    r.n_photons = e.src.photons;
    r.hits = (status == NTP_OK && e.placed) ? s->d_arena + e.offset : nullptr;
    r.t_submit = e.t_submit;
    r.t_launch = e.t_launch;
    r.t_done = e.t_done;
    r.reruns = e.reruns;
    r.batch_events = e.batch_events;
    s->ready.push_back(r);
    ++s->n_completed;
}

// Reads a finished batch.  An event whose last chunk ran completes or, on a
// reservation overflow, goes back to the head of the queue with the exact
// size (to run again from its first photon); an event with photons left goes
// back to the head of the queue too, behind those, for its next chunk: events
// keep their arrival order (the tail latency of a large event is its own
// chunks, not the queue behind it), and every batch still has room for the
// events that arrived meanwhile (a chunk is at most half a batch).
void collect(ntp_server* s, Slot& sl) {
    const unsigned long long* counts = at<const unsigned long long>(sl.h_out, s->off_count);
    std::vector<uint32_t> rerun, cont;
    for (size_t i = 0; i < sl.events.size(); ++i) {
        Event& e = s->events[sl.events[i]];
        e.in_flight = false;
        if (e.launched < e.src.photons) {
            e.state = State::Queued;
            cont.push_back(e.id);
            continue;
        }
        const uint64_t n = counts[i];
        if (n > e.reserve) {
            s->arena.release(e.offset, e.reserve);
            e.placed = false;
            e.reserve = n;
            e.launched = 0;
            ++e.reruns;
            e.state = State::Queued;
            rerun.push_back(e.id);
        } else {
            e.n_hits = n;
            finish_event(s, e, NTP_OK);
        }
    }
    for (auto it = cont.rbegin(); it != cont.rend(); ++it) s->queue.push_front(*it);
    for (auto it = rerun.rbegin(); it != rerun.rend(); ++it) s->queue.push_front(*it);
    sl.events.clear();
    sl.busy = false;
}

// Admits queued events (whole, or their next chunk) into an idle slot and
// launches its graph.
bool launch(ntp_server* s, Slot& sl) {
    auto* hdr = at<uint32_t>(sl.h_in, s->off_hdr);
    auto* src = at<ntp_source>(sl.h_in, s->off_src);
    auto* prefix = at<unsigned long long>(sl.h_in, s->off_prefix);
    auto* stream_ids = at<uint32_t>(sl.h_in, s->off_stream);
    auto* poff = at<unsigned long long>(sl.h_in, s->off_poff);
    auto* outs = at<uint32_t>(sl.h_in, s->off_out);
    auto* nslot = at<uint32_t>(sl.h_in, s->off_nslot);
    auto* nbase = at<unsigned long long>(sl.h_in, s->off_nbase);
    auto* ncap = at<unsigned long long>(sl.h_in, s->off_ncap);
    const uint64_t chunk_max = s->cfg.chunk_photons;
    int k = 0, n_new = 0;
    unsigned long long total = 0;
    prefix[0] = 0;
    const double t = s->now();
    while (!s->queue.empty() && k < s->n_max && total < s->cfg.max_batch_photons) {
        Event& e = s->events[s->queue.front()];
        if (e.src.photons == 0) {  // nothing to simulate
            s->queue.pop_front();
            e.launched = 0;
            finish_event(s, e, NTP_OK);
            continue;
        }
        if (!e.placed) {
            if (e.reserve > s->arena.size()) {  // can never fit
                s->queue.pop_front();
                finish_event(s, e, NTP_ERR_NOMEM);
                continue;
            }
            if (e.out < 0 && s->free_out.empty()) break;  // every output slot in use
            uint64_t off = 0;
            if (!s->arena.alloc(e.reserve, &off)) break;  // wait for releases (FIFO)
            if (e.out < 0) {
                e.out = s->free_out.back();
                s->free_out.pop_back();
            }
            e.offset = off;
            e.placed = true;
            nslot[n_new] = static_cast<uint32_t>(e.out);
            nbase[n_new] = e.offset;
            ncap[n_new] = e.reserve;
            ++n_new;
        }
        uint64_t take = e.src.photons - e.launched;
        if (chunk_max > 0) {
            take = std::min<uint64_t>(take, chunk_max);
            if (k > 0) take = std::min<uint64_t>(take, s->cfg.max_batch_photons - total);
        }
        s->queue.pop_front();
        src[k] = e.src;
        src[k].photons = take;
        stream_ids[k] = e.id;
        poff[k] = e.launched;
        outs[k] = static_cast<uint32_t>(e.out);
        if (e.launched == 0 && e.reruns == 0) e.t_launch = t;
        e.launched += take;
        e.in_flight = true;
        total += take;
        prefix[k + 1] = total;
        sl.events.push_back(e.id);
        ++k;
    }
    if (k == 0) return true;
    hdr[0] = static_cast<uint32_t>(k);
    hdr[1] = static_cast<uint32_t>(n_new);
    for (uint32_t id : sl.events) {
        Event& e = s->events[id];
        e.state = State::Running;
        e.batch_events = std::max(e.batch_events, k);
    }
    ntp::PropParams p;
    fill_slot_params(s, sl, p);
    p.n_src = k;
    p.total = total;
    const unsigned long long warps = static_cast<unsigned long long>(s->grid) * (ntp::kPropBlock / 32);
    unsigned long long chunk = total / (warps * 8);
    chunk = std::max<unsigned long long>(32, std::min<unsigned long long>(4096, chunk));
    p.chunk = (chunk + 31) / 32 * 32;
    cudaKernelNodeParams kp{};
    kp.func = const_cast<void*>(ntp::propagate_kernel_fn());
    kp.gridDim = dim3(s->grid);
    kp.blockDim = dim3(ntp::kPropBlock);
    kp.sharedMemBytes = static_cast<unsigned>(s->smem);
    void* args[] = {&p};
    kp.kernelParams = args;
    if (fail_cuda(s, cudaGraphExecKernelNodeSetParams(sl.exec, sl.kernel_node, &kp), "cudaGraphExecKernelNodeSetParams"))
        return false;
    if (fail_cuda(s, cudaGraphLaunch(sl.exec, sl.stream), "cudaGraphLaunch")) return false;
    if (fail_cuda(s, cudaEventRecord(sl.done, sl.stream), "cudaEventRecord")) return false;
    sl.busy = true;
    ++s->n_batches;
    s->n_photons += total;
    return true;
}

// One pass of the loop; false on a CUDA error.
bool progress(ntp_server* s) {
    for (Slot& sl : s->slots) {
        if (!sl.busy) continue;
        const cudaError_t e = cudaEventQuery(sl.done);
        if (e == cudaSuccess) collect(s, sl);
        else if (e != cudaErrorNotReady) return !fail_cuda(s, e, "cudaEventQuery");
    }
    for (Slot& sl : s->slots)
        if (!sl.busy && !s->queue.empty())
            if (!launch(s, sl)) return false;
    return true;
}

void destroy_slot(Slot& sl) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.exec) cudaGraphExecDestroy(sl.exec);
    if (sl.graph) cudaGraphDestroy(sl.graph);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.d_in) cudaFree(sl.d_in);
    if (sl.d_out) cudaFree(sl.d_out);
    if (sl.h_in) cudaFreeHost(sl.h_in);
    if (sl.h_out) cudaFreeHost(sl.h_out);
    if (sl.stream) cudaStreamDestroy(sl.stream);
}

}  // namespace

extern "C" {

ntp_status ntp_server_create(ntp_ctx* ctx, const ntp_server_config* cfg, ntp_server** out) {
    if (!ctx || !cfg || !out) return NTP_ERR_INVALID;
    *out = nullptr;
    if (cfg->max_events_per_batch < 1 || cfg->max_events_per_batch > 65536 || cfg->max_steps < 1 ||
        cfg->max_steps > (1 << 24) ||
        (cfg->hit_policy != NTP_HIT_FIRST_IN_LIST && cfg->hit_policy != NTP_HIT_NEAREST) ||
        !(cfg->reserve_hits_per_photon >= 0.0) || cfg->hbm_budget_bytes < 64 || cfg->max_batch_photons == 0) {
        ntp::set_ctx_error(ctx, "ntp_server_create: bad configuration");
        return NTP_ERR_INVALID;
    }
    ntp_server* s = new ntp_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    s->t0 = std::chrono::steady_clock::now();
    if (!ntp::fill_world_params(ctx, s->world)) {
        ntp::set_ctx_error(ctx, "ntp_server_create: medium, spectrum and targets must be set first");
        delete s;
        return NTP_ERR_NOT_READY;
    }
    s->world.max_steps = cfg->max_steps;
    s->world.hit_policy = cfg->hit_policy;
    s->world.exact_pole = (cfg->flags & NTP_FLAG_EXACT_POLE_ROTATION) ? 1 : 0;
    if (cfg->flags & NTP_FLAG_PLAIN_SCAN) {
        s->world.columns = nullptr;
        s->world.cell_start = nullptr;
    }
    ntp::set_key(s->world, cfg->seed);
    s->world.refill_min = 8;
    s->n_max = cfg->max_events_per_batch;
    const size_t N = static_cast<size_t>(s->n_max);
    s->off_hdr = 0;
    s->off_src = 16;
    s->off_prefix = align8(s->off_src + sizeof(ntp_source) * N);
    s->off_stream = align8(s->off_prefix + sizeof(unsigned long long) * (N + 1));
    s->off_poff = align8(s->off_stream + sizeof(uint32_t) * N);
    s->off_out = align8(s->off_poff + sizeof(unsigned long long) * N);
    s->off_nslot = align8(s->off_out + sizeof(uint32_t) * N);
    s->off_nbase = align8(s->off_nslot + sizeof(uint32_t) * N);
    s->off_ncap = align8(s->off_nbase + sizeof(unsigned long long) * N);
    s->in_bytes = align8(s->off_ncap + sizeof(unsigned long long) * N);
    s->free_out.reserve(kOutSlots);
    for (int i = kOutSlots - 1; i >= 0; --i) s->free_out.push_back(i);
    s->off_count = 0;
    s->off_counters = align8(sizeof(unsigned long long) * N);
    s->out_bytes = s->off_counters + 4 * sizeof(unsigned long long);

    cudaSetDevice(ntp::ctx_device(ctx));
    auto bail = [&](cudaError_t e, const char* what) {
        fail_cuda(s, e, what);
        ntp_server_destroy(s);
        return NTP_ERR_CUDA;
    };
    const uint64_t arena_hits = cfg->hbm_budget_bytes / sizeof(ntp_hit);
    cudaError_t e = cudaMalloc(&s->d_arena, arena_hits * sizeof(ntp_hit));
    if (e != cudaSuccess) {
        fail_cuda(s, e, "ntp_server_create: arena cudaMalloc");
        ntp_server_destroy(s);
        return NTP_ERR_NOMEM;
    }
    s->arena = Arena(arena_hits);
    if ((e = cudaMalloc(&s->d_ev, 3 * sizeof(unsigned long long) * kOutSlots)) != cudaSuccess)
        return bail(e, "cudaMalloc");
    if ((e = cudaMemset(s->d_ev, 0, 3 * sizeof(unsigned long long) * kOutSlots)) != cudaSuccess)
        return bail(e, "cudaMemset");
    ntp::PropParams probe;
    fill_slot_params(s, s->slots[0], probe);
    int per_sm = 0;
    if ((e = ntp::propagate_occupancy(probe, &per_sm)) != cudaSuccess) return bail(e, "propagate_occupancy");
    if (per_sm < 1) {
        ntp::set_ctx_error(ctx, "ntp_server_create: kernel does not fit on an SM");
        ntp_server_destroy(s);
        return NTP_ERR_INVALID;
    }
    s->grid = per_sm * ntp::ctx_num_sms(ctx);
    s->smem = ntp::prop_smem_bytes(probe);
    for (Slot& sl : s->slots) {
        if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess)
            return bail(e, "cudaStreamCreate");
        if ((e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming)) != cudaSuccess)
            return bail(e, "cudaEventCreate");
        if ((e = cudaMalloc(&sl.d_in, s->in_bytes)) != cudaSuccess) return bail(e, "cudaMalloc");
        if ((e = cudaMalloc(&sl.d_out, s->out_bytes)) != cudaSuccess) return bail(e, "cudaMalloc");
        if ((e = cudaMallocHost(&sl.h_in, s->in_bytes)) != cudaSuccess) return bail(e, "cudaMallocHost");
        if ((e = cudaMallocHost(&sl.h_out, s->out_bytes)) != cudaSuccess) return bail(e, "cudaMallocHost");
        std::memset(sl.h_in, 0, s->in_bytes);
        if (!capture_slot(s, sl)) {
            ntp_server_destroy(s);
            return NTP_ERR_CUDA;
        }
    }
    *out = s;
    return NTP_OK;
}

void ntp_server_destroy(ntp_server* s) {
    if (!s) return;
    cudaSetDevice(ntp::ctx_device(s->ctx));
    for (Slot& sl : s->slots) destroy_slot(sl);
    if (s->d_arena) cudaFree(s->d_arena);
    if (s->d_ev) cudaFree(s->d_ev);
    delete s;
}

ntp_status ntp_server_submit(ntp_server* s, uint32_t event_id, const ntp_source* src) {
    if (!s || !src) return NTP_ERR_INVALID;
    if (s->events.count(event_id)) {
        ntp::set_ctx_error(s->ctx, "ntp_server_submit: event id already pending or not released");
        return NTP_ERR_INVALID;
    }
    if (src->kind < NTP_SRC_POINT_ISOTROPIC || src->kind > NTP_SRC_CHERENKOV_TRACK ||
        (src->kind == NTP_SRC_EXTENDED_CHERENKOV && src->photons > 0 &&
         (!(src->long_a > 1.0f) || !(src->long_b > 0.0f) || !(src->long_lrad > 0.0f)))) {
        ntp::set_ctx_error(s->ctx, "ntp_server_submit: bad source");
        return NTP_ERR_INVALID;
    }
    Event e;
    e.id = event_id;
    e.src = *src;
    e.t_submit = s->now();
    const double want = std::ceil(static_cast<double>(src->photons) * s->cfg.reserve_hits_per_photon);
    e.reserve = std::max<uint64_t>(s->cfg.min_reserve_hits, static_cast<uint64_t>(want));
    s->events.emplace(event_id, e);
    s->queue.push_back(event_id);
    return NTP_OK;
}

int32_t ntp_server_poll(ntp_server* s, ntp_event_result* out, int32_t max, int32_t timeout_us) {
    if (!s || (max > 0 && !out)) return -1;
    cudaSetDevice(ntp::ctx_device(s->ctx));
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::microseconds(std::max(0, timeout_us));
    for (;;) {
        if (!progress(s)) return -1;
        if (!s->ready.empty() || max == 0) break;
        const bool busy = s->slots[0].busy || s->slots[1].busy;
        if (!busy && s->queue.empty()) break;
        if (std::chrono::steady_clock::now() >= deadline) break;
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    int32_t n = 0;
    while (n < max && !s->ready.empty()) {
        out[n++] = s->ready.front();
        s->ready.pop_front();
    }
    return n;
}

ntp_status ntp_server_copy_hits(ntp_server* s, uint32_t event_id, ntp_hit* dst, uint64_t max, uint64_t* n) {
    if (!s || (max > 0 && !dst)) return NTP_ERR_INVALID;
    auto it = s->events.find(event_id);
    if (it == s->events.end() || it->second.state != State::Done) {
        ntp::set_ctx_error(s->ctx, "ntp_server_copy_hits: event is not finished");
        return NTP_ERR_INVALID;
    }
    const Event& e = it->second;
    if (n) *n = e.n_hits;
    const uint64_t k = std::min<uint64_t>(max, e.placed ? e.n_hits : 0);
    if (k == 0) return NTP_OK;
    cudaSetDevice(ntp::ctx_device(s->ctx));
    if (fail_cuda(s, cudaMemcpy(dst, s->d_arena + e.offset, k * sizeof(ntp_hit), cudaMemcpyDeviceToHost),
                  "cudaMemcpy"))
        return NTP_ERR_CUDA;
    return NTP_OK;
}

ntp_status ntp_server_release(ntp_server* s, uint32_t event_id) {
    if (!s) return NTP_ERR_INVALID;
    auto it = s->events.find(event_id);
    if (it == s->events.end() || it->second.state != State::Done) {
        ntp::set_ctx_error(s->ctx, "ntp_server_release: event is not finished");
        return NTP_ERR_INVALID;
    }
    if (it->second.placed) s->arena.release(it->second.offset, it->second.reserve);
    s->events.erase(it);
    ++s->n_released;
    return NTP_OK;
}

ntp_status ntp_server_get_stats(const ntp_server* s, ntp_server_stats* out) {
    if (!s || !out) return NTP_ERR_INVALID;
    ntp_server_stats st{};
    st.queued = s->queue.size();
    for (const Slot& sl : s->slots) st.running += sl.events.size();
    // events between chunks wait in the queue: count them as running
    for (uint32_t id : s->queue) {
        auto it = s->events.find(id);
        if (it != s->events.end() && it->second.launched > 0) {
            --st.queued;
            ++st.running;
        }
    }
    st.completed = s->n_completed;
    st.released = s->n_released;
    st.batches = s->n_batches;
    st.photons = s->n_photons;
    st.arena_hits = s->arena.size();
    st.arena_reserved_hits = s->arena.used();
    st.clock = s->now();
    *out = st;
    return NTP_OK;
}

}  // extern "C"
