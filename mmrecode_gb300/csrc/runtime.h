// Host runtime around the decode engines: a pool that splits large batches over
// several engines (each its own CUDA stream and device arenas) so that host
// planning, uploads, kernels and read-backs of different chunks overlap, and a
// serving loop that admits requests from many streams against a device-memory
// budget and batches them continuously.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "engine.h"

namespace mmr {

// Sum of per-chunk stage times (device work) and counters of one pooled decode.
void accumulate_times(EngineTimes &into, const EngineTimes &t);

// One tuned class: the slice size chosen for it and the entropy-stage time of
// every candidate on the sample (ms, best of the repetitions).
// One class of the autotuner's table. kind 0: slice bits of an entropy class
// (ms = entropy stage per candidate slice size); kind 1: strip of a transform
// tiling class (strip_mcus = chosen MCUs per CTA, ms[0..1] = transform stage
// with the narrow and the wide strip).
struct TuneResult {
    uint32_t kind = 0;
    uint32_t frame_class = 0;
    uint32_t slice_bits = 0;
    uint32_t strip_mcus = 0;
    uint32_t frames = 0;
    double ms[4] = {0, 0, 0, 0};
};
constexpr uint32_t kTuneCandidates[4] = {1024, 2048, 4096, 8192};

class EnginePool {
public:
    EnginePool(int device, int engines);
    ~EnginePool();
    EnginePool(const EnginePool &) = delete;
    EnginePool &operator=(const EnginePool &) = delete;

    // Decodes the items; batches of at least 2 * min_chunk items are split into
    // chunks decoded concurrently by all engines. Outputs in host memory (and
    // packets in host memory) are staged through device buffers: a chunk's
    // packets go up on its engine's stream, the chunk decodes device-resident (and replays as a graph when it
    // repeats), and its outputs come down on the engine's download stream while
    // the engine takes its next chunk. Staged chunk i runs at stream priority
    // level i, so concurrent chunks finish in order and their downloads spread
    // over the batch instead of queueing at its end. times: stage times summed
    // over chunks, device_ms = wall time of the call. Returns kOk or kInternal.
    int32_t decode(Item *items, size_t n, EngineTimes *times);
    uint32_t last_launches() const { return launches_; }
    bool set_slice_bits(uint32_t bits);
    void set_graphs(bool on);
    // Measures the entropy stage of the sample's MJPEG frames, class by class, at
    // every candidate slice size, and the fused transform of its RGB24 frames,
    // tiling class by class, with the narrow and the wide strip, on one engine,
    // and keeps the fastest per class for all engines (classes not in the sample
    // keep the automatic choice). Decodes the items (outputs included) several
    // times.
    std::vector<TuneResult> autotune(Item *items, size_t n);
    // Installs a table (from autotune, or saved from an earlier one) on all engines.
    void set_tuning(const std::vector<TuneResult> &table);
    int size() const { return (int)engines_.size(); }
    int device() const { return device_; }
    Engine &engine(int k) { return *engines_[k]; }
    static constexpr size_t kMinChunk = 16;

private:
    struct Chunk {
        Item *items;
        size_t n;
        EngineTimes times;
        uint32_t launches;
        int32_t status;
        size_t first;  // index of items[0] in the batch
    };
    void worker(int k);
    // Redirects host payloads of the batch to device staging buffers (into
    // staged_); false when nothing was redirected.
    bool stage(const Item *items, size_t n);
    std::vector<std::unique_ptr<Engine>> engines_;
    std::vector<cudaStream_t> down_;  // per engine: downloads of staged outputs
    int device_ = 0;
    // staging of the current batch: device copies of its inputs and outputs
    void *stage_ptr_ = nullptr;
    size_t stage_cap_ = 0;
    std::vector<Item> staged_;
    std::vector<uint8_t> redirected_;  // per item: kStagedIn | kStagedOut
    static constexpr uint8_t kStagedIn = 1;   // the packet goes up through the staging buffer
    static constexpr uint8_t kStagedOut = 2;  // the output comes down from it
    const Item *orig_ = nullptr;       // the caller's items of the current batch
    std::vector<std::thread> threads_;
    std::mutex call_mu_;  // one decode call at a time
    std::mutex mu_;
    std::condition_variable work_cv_, done_cv_;
    std::vector<Chunk> chunks_;
    size_t done_ = 0;
    uint64_t gen_ = 0;  // batches handed to the workers
    bool stop_ = false;
    uint32_t launches_ = 0;
    std::map<uint32_t, uint32_t> tuned_;       // entropy class -> slice bits
    std::map<uint32_t, uint32_t> tuned_tile_;  // tiling class -> wide strip (1) or narrow (0)
};

struct ServerConfig {
    int device = 0;
    int engines = 3;
    size_t max_batch = 64;
    uint64_t memory_budget = 0;  // device bytes for all batches in flight; 0 = no cap
};

struct ServerStats {
    uint64_t submitted = 0, completed = 0, failed = 0, rejected = 0, batches = 0;
    uint64_t in_flight = 0, queued = 0;
    double p50_ms = 0, p99_ms = 0, max_ms = 0, mean_ms = 0;
    double frames_per_s = 0;   // completed over the window
    double window_s = 0;       // since creation or the last reset
    uint64_t peak_budget_bytes = 0;  // largest estimated footprint of the batches in flight
};

// Continuous batching: requests queue as they arrive; each engine's worker takes
// the oldest requests that fit its share of the memory budget (and max_batch),
// decodes them, completes them and takes the next ones, so requests that arrive
// while others are on the GPU join the next free batch.
class Server {
public:
    struct Request {
        Item item;
        uint64_t ticket = 0;
        uint64_t est_bytes = 0;
        std::chrono::steady_clock::time_point submitted;
        double latency_ms = 0;
        bool done = false;
    };

    explicit Server(const ServerConfig &cfg);
    ~Server();
    Server(const Server &) = delete;
    Server &operator=(const Server &) = delete;

    // Queues a copy of the item (its data and output buffers stay the caller's
    // until completion). Returns 0 and sets the ticket, or a status when the
    // request alone exceeds an engine's share of the budget.
    int32_t submit(const Item &item, uint64_t *ticket);
    // Waits up to timeout_ns (< 0: forever) for the ticket; on completion copies
    // the result into *out and forgets the ticket. Returns false on timeout.
    bool wait(uint64_t ticket, int64_t timeout_ns, Item *out, double *latency_ms);
    bool known(uint64_t ticket);
    ServerStats stats(bool reset);
    bool set_slice_bits(uint32_t bits);
    // Installs an autotuner table on the server's engines (later batches use it).
    void set_tuning(const std::vector<TuneResult> &table);
    // Open-loop trace replay: submits item i at arrival_ns[i] after the call starts
    // (non-decreasing offsets), collects every result into items[i] and its latency
    // into latency_ms[i]; *max_lag_ns = the latest any submission left its slot.
    // Items the budget refuses complete at once with kInvalidArgument.
    void replay(Item *items, size_t n, const int64_t *arrival_ns, double *latency_ms, int64_t *max_lag_ns);

    // Device bytes a request needs inside a batch (inputs, outputs, coefficient
    // and slice arenas), from its headers.
    static uint64_t estimate_bytes(const Item &item);

private:
    void worker(int k);
    ServerConfig cfg_;
    uint64_t share_ = 0;  // budget per engine
    std::vector<std::unique_ptr<Engine>> engines_;
    std::vector<std::thread> threads_;
    std::mutex mu_;
    std::condition_variable work_cv_, done_cv_;
    std::deque<std::shared_ptr<Request>> queue_;
    std::unordered_map<uint64_t, std::shared_ptr<Request>> live_;  // submitted, not yet collected
    uint64_t next_ticket_ = 1;
    bool stop_ = false;
    uint64_t in_flight_ = 0, in_flight_bytes_ = 0;
    ServerStats totals_;
    std::vector<double> lat_;  // latencies of completed requests in the window
    std::chrono::steady_clock::time_point window_start_;
};

}  // namespace mmr
