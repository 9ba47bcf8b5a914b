// Host runtime: engine pool for large batches and the continuous-batching server.
#include "runtime.h"

#include <algorithm>
#include <chrono>
#include <stdexcept>

namespace mmr {

void accumulate_times(EngineTimes &a, const EngineTimes &t) {
    a.upload_ms += t.upload_ms;
    a.scan_ms += t.scan_ms;
    a.entropy_ms += t.entropy_ms;
    a.idct_ms += t.idct_ms;
    a.dv_ms += t.dv_ms;
    a.rgb_ms += t.rgb_ms;
    a.download_ms += t.download_ms;
    a.slice_spec_ms += t.slice_spec_ms;
    a.slice_sync_ms += t.slice_sync_ms;
    a.slice_decode_ms += t.slice_decode_ms;
    a.dv_segment_ms += t.dv_segment_ms;
    a.dv_idct_ms += t.dv_idct_ms;
    a.input_bytes += t.input_bytes;
    a.output_bytes += t.output_bytes;
    a.jpeg_blocks += t.jpeg_blocks;
    a.dv_blocks += t.dv_blocks;
    a.rgb_pixels += t.rgb_pixels;
    a.idct_exact_samples += t.idct_exact_samples;
    a.graph_replays += t.graph_replays;
    a.slices += t.slices;
    a.slices_redone += t.slices_redone;
    a.slices_redone_whole += t.slices_redone_whole;
}

// ------------------------------------------------------------------ pool ---

EnginePool::EnginePool(int device, int engines) : device_(device) {
    engines = std::max(1, engines);
    for (int k = 0; k < engines; k++) {
        // chunk i of a batch runs at priority level i: chunks complete in order
        engines_.emplace_back(new Engine(device, engines > 1 ? 2 * engines : 1));
        cudaStream_t d = nullptr;
        if (cudaStreamCreateWithFlags(&d, cudaStreamNonBlocking) != cudaSuccess)
            throw std::runtime_error("cannot create a download stream");
        down_.push_back(d);
    }
    for (int k = 0; k < engines; k++) threads_.emplace_back(&EnginePool::worker, this, k);
}

EnginePool::~EnginePool() {
    {
        std::lock_guard<std::mutex> g(mu_);
        stop_ = true;
    }
    work_cv_.notify_all();
    for (auto &t : threads_) t.join();
    cudaSetDevice(device_);
    for (cudaStream_t d : down_) {
        cudaStreamSynchronize(d);
        cudaStreamDestroy(d);
    }
    if (stage_ptr_) cudaFree(stage_ptr_);
}

bool EnginePool::stage(const Item *items, size_t n) {
    staged_.assign(items, items + n);
    redirected_.assign(n, 0);
    orig_ = items;
    std::vector<size_t> in_off(n), out_off(n);
    size_t total = 0;
    bool any = false;
    for (size_t i = 0; i < n; i++) {
        const Item &it = items[i];
        // single-buffer host outputs (planes written to separate pointers stay on the
        // engine's path), with their packets when those are in host memory too
        if (it.out_on_device || !it.out || !it.out_capacity || it.plane_out[0]) continue;
        if (!it.dev_data && (!it.data || !it.len)) continue;
        redirected_[i] = kStagedOut;
        any = true;
        if (!it.dev_data) {
            redirected_[i] |= kStagedIn;
            in_off[i] = total;
            total += (it.len + 255) / 256 * 256;
        }
        out_off[i] = total;
        total += (it.out_capacity + 255) / 256 * 256;
    }
    if (!any) return false;
    if (total > stage_cap_) {
        const size_t want = std::max(total, stage_cap_ + stage_cap_ / 2);
        if (stage_ptr_) cudaFree(stage_ptr_);
        stage_ptr_ = nullptr;
        stage_cap_ = 0;
        if (cudaMalloc(&stage_ptr_, want) != cudaSuccess) {  // no room: the engines copy directly
            cudaGetLastError();
            stage_ptr_ = nullptr;
            return false;
        }
        stage_cap_ = want;
    }
    uint8_t *base = static_cast<uint8_t *>(stage_ptr_);
    for (size_t i = 0; i < n; i++) {
        if (!redirected_[i]) continue;
        if (redirected_[i] & kStagedIn) staged_[i].dev_data = base + in_off[i];
        staged_[i].out = base + out_off[i];
        staged_[i].out_on_device = true;
    }
    return true;
}

void EnginePool::set_graphs(bool on) {
    for (auto &e : engines_) e->set_graphs(on);
}

bool EnginePool::set_slice_bits(uint32_t bits) {
    bool ok = true;
    for (auto &e : engines_) ok &= e->set_slice_bits(bits);
    return ok;
}

// Worker k decodes chunks k, k + K, k + 2K, ... of each batch: a repeated batch
// meets the same engine chunk by chunk, so its graphs replay.
void EnginePool::worker(int k) {
    uint64_t seen = 0;
    for (;;) {
        std::unique_lock<std::mutex> lk(mu_);
        work_cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
        if (stop_) return;
        seen = gen_;
        const size_t n_chunks = chunks_.size();
        const bool staging = !redirected_.empty();
        lk.unlock();
        Engine &e = *engines_[k];
        for (size_t i = k; i < n_chunks; i += engines_.size()) {
            Chunk &c = chunks_[i];
            e.set_level(staging ? (int)i : 0);  // staged chunks complete in order, for their downloads
            c.status = kOk;
            if (staging) {  // inputs up, ahead of the chunk's kernels on the same stream
                for (size_t j = 0; j < c.n && c.status == kOk; j++)
                    if ((redirected_[c.first + j] & kStagedIn) &&
                        cudaMemcpyAsync(const_cast<uint8_t *>(c.items[j].dev_data), c.items[j].data, c.items[j].len,
                                        cudaMemcpyHostToDevice, e.stream()) != cudaSuccess)
                        c.status = kInternal;
            }
            if (c.status == kOk) {
                c.status = e.decode(c.items, c.n, &c.times);
                c.launches = e.last_launches();
            }
            if (staging && c.status == kOk) {  // outputs down, while this engine takes its next chunk
                for (size_t j = 0; j < c.n && c.status == kOk; j++) {
                    const Item &it = c.items[j];
                    if ((redirected_[c.first + j] & kStagedOut) && it.status == kOk && it.out_bytes &&
                        cudaMemcpyAsync(orig_[c.first + j].out, it.out, it.out_bytes, cudaMemcpyDeviceToHost,
                                        down_[k]) != cudaSuccess)
                        c.status = kInternal;
                }
            }
            if (c.status != kOk) {
                cudaGetLastError();
                for (size_t j = 0; j < c.n; j++) {
                    c.items[j].diag = make_diag(kDeviceError);
                    c.items[j].status = kInternal;
                    if (c.items[j].message.empty()) c.items[j].message = "CUDA device failure: staging copy";
                    c.items[j].out_bytes = 0;
                }
            }
            lk.lock();
            if (++done_ == n_chunks) done_cv_.notify_all();
            lk.unlock();
        }
    }
}

std::vector<TuneResult> EnginePool::autotune(Item *items, size_t n) {
    std::lock_guard<std::mutex> call(call_mu_);
    std::map<uint32_t, std::vector<Item>> classes, tiles;
    for (size_t i = 0; i < n; i++) {
        if (items[i].codec != kCodecMjpeg) continue;
        const uint32_t c = jpeg_tune_class(items[i].data, items[i].len);
        if (c != 0xffffffffu && classes[c].size() < 64) classes[c].push_back(items[i]);
        if (items[i].output != kOutRgb24) continue;
        const uint32_t t = jpeg_tile_class(items[i].data, items[i].len);
        if (t != 0xffffffffu && tiles[t].size() < 64) tiles[t].push_back(items[i]);
    }
    Engine &e = *engines_[0];
    e.set_level(0);
    const uint32_t keep_bits = e.slice_bits();
    // best of three timed runs (the first run sizes the arenas and is not counted)
    auto best_of = [&](std::vector<Item> &v, float EngineTimes::*stage) {
        double m = 1e30;
        for (int rep = 0; rep < 3; rep++) {
            EngineTimes t;
            e.decode(v.data(), v.size(), &t);
            if (rep) m = std::min(m, (double)(t.*stage));
        }
        return m;
    };
    std::vector<TuneResult> out;
    for (auto &kv : classes) {
        TuneResult r;
        r.kind = 0;
        r.frame_class = kv.first;
        r.frames = (uint32_t)kv.second.size();
        double best = 1e30;
        for (int k = 0; k < 4; k++) {
            e.set_slice_bits(kTuneCandidates[k]);
            r.ms[k] = best_of(kv.second, &EngineTimes::entropy_ms);
            if (r.ms[k] < best) {
                best = r.ms[k];
                r.slice_bits = kTuneCandidates[k];
            }
        }
        tuned_[kv.first] = r.slice_bits;
        out.push_back(r);
    }
    e.set_slice_bits(keep_bits);
    e.set_tuned(tuned_);
    for (auto &kv : tiles) {
        TuneResult r;
        r.kind = 1;
        r.frame_class = kv.first;
        r.frames = (uint32_t)kv.second.size();
        for (int wide = 0; wide < 2; wide++) {
            e.set_fused_wide(wide);
            r.ms[wide] = best_of(kv.second, &EngineTimes::idct_ms);
        }
        const int wide = r.ms[1] <= r.ms[0] ? 1 : 0;
        r.strip_mcus = fused_strip_mcus(kv.first, wide != 0);
        tuned_tile_[kv.first] = (uint32_t)wide;
        out.push_back(r);
    }
    e.set_fused_wide(-1);
    for (auto &en : engines_) {
        en->set_tuned(tuned_);
        en->set_tuned_tiles(tuned_tile_);
    }
    return out;
}

void EnginePool::set_tuning(const std::vector<TuneResult> &table) {
    std::lock_guard<std::mutex> call(call_mu_);
    for (const TuneResult &r : table) {
        if (r.kind == 0) {
            tuned_[r.frame_class] = r.slice_bits;
        } else {
            tuned_tile_[r.frame_class] = r.strip_mcus == fused_strip_mcus(r.frame_class, true) ? 1u : 0u;
        }
    }
    for (auto &en : engines_) {
        en->set_tuned(tuned_);
        en->set_tuned_tiles(tuned_tile_);
    }
}

int32_t EnginePool::decode(Item *items, size_t n, EngineTimes *times) {
    std::lock_guard<std::mutex> call(call_mu_);
    const auto t0 = std::chrono::steady_clock::now();
    const size_t k = engines_.size();
    int32_t status;
    EngineTimes sum;
    if (k == 1 || n < 2 * kMinChunk) {
        // small batch: the calling thread decodes on the first engine
        engines_[0]->set_level(0);
        status = engines_[0]->decode(items, n, &sum);
        launches_ = engines_[0]->last_launches();
    } else {
        // two chunks per engine: each engine plans its next chunk while its last
        // one is on the GPU next to the other engines' chunks
        const size_t parts = std::min(2 * k, n / kMinChunk);
        Item *work = items;
        if (cudaSetDevice(device_) == cudaSuccess && stage(items, n)) work = staged_.data();
        else redirected_.clear();
        std::unique_lock<std::mutex> lk(mu_);
        chunks_.clear();
        for (size_t p = 0, first = 0; p < parts; p++) {
            const size_t cnt = n / parts + (p < n % parts ? 1 : 0);
            chunks_.push_back({work + first, cnt, EngineTimes(), 0, kOk, first});
            first += cnt;
        }
        done_ = 0;
        gen_++;
        work_cv_.notify_all();
        done_cv_.wait(lk, [&] { return done_ == chunks_.size(); });
        lk.unlock();
        status = kOk;
        if (work != items) {  // downloads done, results back into the caller's items
            for (cudaStream_t d : down_)
                if (cudaStreamSynchronize(d) != cudaSuccess) status = kInternal;
            cudaGetLastError();
            for (size_t i = 0; i < n; i++) {
                Item &dst = items[i];
                const Item &src = staged_[i];
                const uint8_t *dev = dst.dev_data, *data = dst.data;
                uint8_t *out = dst.out;
                const bool on_device = dst.out_on_device;
                dst = src;
                dst.data = data;
                dst.dev_data = dev;
                dst.out = out;
                dst.out_on_device = on_device;
                if (status != kOk) {
                    dst.diag = make_diag(kDeviceError);
                    dst.status = kInternal;
                    dst.message = "CUDA device failure: staging copy";
                    dst.out_bytes = 0;
                }
            }
            redirected_.clear();
        }
        launches_ = 0;
        for (const Chunk &c : chunks_) {
            accumulate_times(sum, c.times);
            launches_ += c.launches;
            if (c.status != kOk) status = c.status;
        }
    }
    sum.device_ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (times) *times = sum;
    return status;
}

// ---------------------------------------------------------------- server ---

uint64_t Server::estimate_bytes(const Item &it) {
    const Probe p = probe_packet(it.codec, it.data, it.len);
    const uint64_t planar = p.status == kOk ? p.planar_bytes : 0;
    const uint64_t out = p.status == kOk ? (it.output == kOutRgb24 ? p.rgb_bytes : planar) : 0;
    // tokens and slice records (~8 B per compressed byte at the smallest automatic
    // slice), coefficients in place and in the speculative decode's scratch
    // (~4.5 B per sample), planes, fixed scratch
    uint64_t b = 8 * (uint64_t)it.len + (planar * 9) / 2 + planar + 65536;
    if (!it.out_on_device) b += out;  // staged output
    return b;
}

Server::Server(const ServerConfig &cfg) : cfg_(cfg) {
    cfg_.engines = std::max(1, cfg_.engines);
    cfg_.max_batch = std::max<size_t>(1, cfg_.max_batch);
    share_ = cfg_.memory_budget ? cfg_.memory_budget / cfg_.engines : 0;
    window_start_ = std::chrono::steady_clock::now();
    for (int k = 0; k < cfg_.engines; k++) engines_.emplace_back(new Engine(cfg_.device));
    for (int k = 0; k < cfg_.engines; k++) threads_.emplace_back(&Server::worker, this, k);
}

Server::~Server() {
    {
        std::unique_lock<std::mutex> lk(mu_);
        // finish what was submitted
        done_cv_.wait(lk, [&] { return queue_.empty() && in_flight_ == 0; });
        stop_ = true;
    }
    work_cv_.notify_all();
    for (auto &t : threads_) t.join();
}

void Server::set_tuning(const std::vector<TuneResult> &table) {
    std::map<uint32_t, uint32_t> tuned, tiles;
    for (const TuneResult &r : table) {
        if (r.kind == 0) tuned[r.frame_class] = r.slice_bits;
        else tiles[r.frame_class] = r.strip_mcus == fused_strip_mcus(r.frame_class, true) ? 1u : 0u;
    }
    for (auto &e : engines_) {
        e->set_tuned(tuned);
        e->set_tuned_tiles(tiles);
    }
}

bool Server::set_slice_bits(uint32_t bits) {
    std::lock_guard<std::mutex> g(mu_);
    bool ok = true;
    for (auto &e : engines_) ok &= e->set_slice_bits(bits);
    return ok;
}

int32_t Server::submit(const Item &item, uint64_t *ticket) {
    auto r = std::make_shared<Request>();
    r->item = item;
    r->est_bytes = estimate_bytes(item);
    if (share_ && r->est_bytes > share_) {
        std::lock_guard<std::mutex> g(mu_);
        totals_.rejected++;
        return kInvalidArgument;
    }
    r->submitted = std::chrono::steady_clock::now();
    {
        std::lock_guard<std::mutex> g(mu_);
        r->ticket = next_ticket_++;
        live_[r->ticket] = r;
        queue_.push_back(r);
        totals_.submitted++;
    }
    work_cv_.notify_one();
    *ticket = r->ticket;
    return kOk;
}

void Server::worker(int k) {
    Engine &engine = *engines_[k];
    std::vector<std::shared_ptr<Request>> batch;
    std::vector<Item> items;
    for (;;) {
        batch.clear();
        uint64_t bytes = 0;
        {
            std::unique_lock<std::mutex> lk(mu_);
            work_cv_.wait(lk, [&] { return stop_ || !queue_.empty(); });
            if (stop_ && queue_.empty()) return;
            // the oldest requests that fit this engine's share of the budget
            while (!queue_.empty() && batch.size() < cfg_.max_batch) {
                const auto &r = queue_.front();
                if (!batch.empty() && share_ && bytes + r->est_bytes > share_) break;
                bytes += r->est_bytes;
                batch.push_back(r);
                queue_.pop_front();
            }
            in_flight_ += batch.size();
            in_flight_bytes_ += bytes;
            totals_.peak_budget_bytes = std::max(totals_.peak_budget_bytes, in_flight_bytes_);
            totals_.batches++;
            if (!queue_.empty()) work_cv_.notify_one();  // more work for an idle engine
        }
        items.resize(batch.size());
        for (size_t i = 0; i < batch.size(); i++) items[i] = batch[i]->item;
        engine.decode(items.data(), items.size(), nullptr);
        const auto now = std::chrono::steady_clock::now();
        {
            std::lock_guard<std::mutex> g(mu_);
            for (size_t i = 0; i < batch.size(); i++) {
                Request &r = *batch[i];
                r.item = items[i];
                r.latency_ms = std::chrono::duration<double, std::milli>(now - r.submitted).count();
                r.done = true;
                lat_.push_back(r.latency_ms);
                totals_.completed++;
                if (r.item.status != kOk) totals_.failed++;
            }
            in_flight_ -= batch.size();
            in_flight_bytes_ -= bytes;
        }
        done_cv_.notify_all();
    }
}

bool Server::wait(uint64_t ticket, int64_t timeout_ns, Item *out, double *latency_ms) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = live_.find(ticket);
    if (it == live_.end()) return false;
    std::shared_ptr<Request> r = it->second;
    auto ready = [&] { return r->done; };
    if (timeout_ns < 0) done_cv_.wait(lk, ready);
    else if (!done_cv_.wait_for(lk, std::chrono::nanoseconds(timeout_ns), ready)) return false;
    if (out) *out = r->item;
    if (latency_ms) *latency_ms = r->latency_ms;
    live_.erase(ticket);
    return true;
}

void Server::replay(Item *items, size_t n, const int64_t *arrival_ns, double *latency_ms, int64_t *max_lag_ns) {
    std::vector<uint64_t> tickets(n, 0);
    std::atomic<size_t> submitted{0};
    std::mutex m;
    std::condition_variable cv;
    std::thread collector([&] {
        for (size_t i = 0; i < n; i++) {
            {
                std::unique_lock<std::mutex> lk(m);
                cv.wait(lk, [&] { return submitted.load() > i; });
            }
            if (tickets[i] == 0) {
                latency_ms[i] = 0;
                continue;
            }
            wait(tickets[i], -1, &items[i], &latency_ms[i]);
        }
    });
    const auto t0 = std::chrono::steady_clock::now();
    int64_t lag = 0;
    for (size_t i = 0; i < n; i++) {
        const auto at = t0 + std::chrono::nanoseconds(arrival_ns[i]);
        std::this_thread::sleep_until(at);
        lag = std::max<int64_t>(lag, std::chrono::duration_cast<std::chrono::nanoseconds>(
                                         std::chrono::steady_clock::now() - at).count());
        uint64_t t = 0;
        if (submit(items[i], &t) != kOk) {
            items[i].status = kInvalidArgument;
            items[i].message = "request exceeds the server's device-memory budget per engine";
        }
        {
            std::lock_guard<std::mutex> g(m);
            tickets[i] = t;
            submitted.store(i + 1);
        }
        cv.notify_one();
    }
    collector.join();
    if (max_lag_ns) *max_lag_ns = lag;
}

bool Server::known(uint64_t ticket) {
    std::lock_guard<std::mutex> g(mu_);
    return live_.count(ticket) != 0;
}

ServerStats Server::stats(bool reset) {
    std::lock_guard<std::mutex> g(mu_);
    ServerStats s = totals_;
    s.in_flight = in_flight_;
    s.queued = queue_.size();
    const auto now = std::chrono::steady_clock::now();
    s.window_s = std::chrono::duration<double>(now - window_start_).count();
    if (!lat_.empty()) {
        std::vector<double> v(lat_);
        std::sort(v.begin(), v.end());
        auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * v.size()))]; };
        s.p50_ms = pct(0.50);
        s.p99_ms = pct(0.99);
        s.max_ms = v.back();
        double sum = 0;
        for (double x : v) sum += x;
        s.mean_ms = sum / v.size();
        s.frames_per_s = s.window_s > 0 ? v.size() / s.window_s : 0;
    }
    if (reset) {  // counters and latencies start again
        lat_.clear();
        window_start_ = now;
        totals_ = ServerStats();
        totals_.peak_budget_bytes = in_flight_bytes_;
    }
    return s;
}

}  // namespace mmr
