// fn_server.cpp -- continuous-batching request server (see fn_server.h).
#include "fn_server.h"

#include "fn_jit.h"

#include <algorithm>
#include <cstring>

namespace fn {

// ------------------------------------------------------------------ pool

bool DevicePool::init(size_t bytes)
{
    bytes = (bytes + 255) & ~(size_t)255;
    if (!cuda_ok(cudaMalloc(&base_, bytes), "cudaMalloc(pool)")) return false;
    cap_ = bytes;
    free_[0] = bytes;
    return true;
}

DevicePool::~DevicePool()
{
    if (base_) cudaFree(base_);
}

bool DevicePool::alloc(size_t bytes, size_t& offset)
{
    bytes = std::max<size_t>(256, (bytes + 255) & ~(size_t)255);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
        if (it->second >= bytes) {
            offset = it->first;
            size_t rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[offset + bytes] = rest;
            live_[offset] = bytes;
            used_ += bytes;
            return true;
        }
    }
    return false;
}

void DevicePool::free(size_t offset)
{
    auto it = live_.find(offset);
    if (it == live_.end()) return;
    size_t size = it->second;
    live_.erase(it);
    used_ -= size;
    auto next = free_.lower_bound(offset);
    if (next != free_.end() && offset + size == next->first) {       // merge right
        size += next->second;
        next = free_.erase(next);
    }
    if (next != free_.begin()) {                                      // merge left
        auto prev = std::prev(next);
        if (prev->first + prev->second == offset) {
            prev->second += size;
            return;
        }
    }
    free_[offset] = size;
}

// ------------------------------------------------------------------ server

Server::Server(const ServerConfig& cfg) : cfg_(cfg)
{
    if (cfg_.streams < 1) cfg_.streams = 1;
    if (cfg_.max_batch_requests < 1) cfg_.max_batch_requests = 1;
    if (!thread_ctx()) return;
    cudaGetDevice(&device_);
    if (!pool_.init(cfg_.pool_bytes)) return;
    n_slots_ = std::max(4096, cfg_.streams * cfg_.max_batch_requests);
    if (!cuda_ok(cudaHostAlloc(&slots_, sizeof(Slot) * n_slots_, cudaHostAllocMapped), "cudaHostAlloc(slots)")) return;
    std::memset(slots_, 0, sizeof(Slot) * n_slots_);
    if (!cuda_ok(cudaHostGetDevicePointer(reinterpret_cast<void**>(&slots_dev_), slots_, 0), "mapped slots")) return;
    for (int i = n_slots_ - 1; i >= 0; --i) free_slots_.push_back(i);
    flights_.resize(cfg_.streams);
    for (auto& f : flights_) {
        if (!cuda_ok(cudaStreamCreateWithFlags(&f.stream, cudaStreamNonBlocking), "stream") ||
            !cuda_ok(cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming), "event"))
            return;
        f.runner.reset(new BatchRunner());
    }
    ok_ = true;
    thread_ = std::thread([this] { loop(); });
}

Server::~Server()
{
    stop_ = true;
    cv_work_.notify_all();
    if (thread_.joinable()) thread_.join();
    for (auto& f : flights_) {
        if (f.stream) { cudaStreamSynchronize(f.stream); cudaStreamDestroy(f.stream); }
        if (f.done) cudaEventDestroy(f.done);
        f.runner.reset();
    }
    for (auto& kv : recs_) {
        if (kv.second.pooled) pool_.free(kv.second.pool_off);
        node_unref(const_cast<Node*>(kv.second.item.node));
    }
    if (slots_) cudaFreeHost(slots_);
}

int Server::validate(const BatchItem& item)
{
    if (!item.node || item.args.total < 0) { set_error(-1, "invalid request"); return -1; }
    DeviceProgram p;                      // compile now so the submitter sees tree errors
    if (!get_program(item.node, item.args.dim, p)) return last_error();
    std::string jerr;                     // and specialise trees the interpreter cannot run
    if (!jit_ensure(p.host, jerr)) { set_error(-2, jerr); return -2; }
    const size_t bytes = (size_t)std::max(0ll, item.args.total) * sizeof(float);
    if (!item.dout && bytes > pool_.capacity()) { set_error(-4, "request output larger than the device pool"); return -4; }
    return 0;
}

int Server::enqueue_locked(const BatchItem& item, std::chrono::steady_clock::time_point t_submit, uint64_t& ticket)
{
    node_ref(const_cast<Node*>(item.node));
    ticket = next_ticket_++;
    Record& r = recs_[ticket];
    r.item = item;
    r.t_submit = t_submit;
    queue_.push_back(ticket);
    ++submitted_;
    return 0;
}

int Server::submit(const BatchItem& item, uint64_t& ticket)
{
    if (!ok_) { set_error(-6, "server is not running"); return -6; }
    if (int rc = validate(item)) return rc;
    std::lock_guard<std::mutex> lk(mu_);
    enqueue_locked(item, std::chrono::steady_clock::now(), ticket);
    cv_work_.notify_one();
    return 0;
}

int Server::submit_paced(const BatchItem* items, size_t n, const double* arrival_us, uint64_t* tickets)
{
    if (!ok_) { set_error(-6, "server is not running"); return -6; }
    for (size_t i = 0; i < n; ++i)
        if (int rc = validate(items[i])) return rc;
    using clock = std::chrono::steady_clock;
    const clock::time_point start = clock::now();
    for (size_t i = 0; i < n; ++i) {
        const clock::time_point due = start + std::chrono::duration_cast<clock::duration>(
                                                  std::chrono::duration<double, std::micro>(arrival_us[i]));
        while (clock::now() < due) {
        }
        std::lock_guard<std::mutex> lk(mu_);
        enqueue_locked(items[i], due, tickets[i]);
        cv_work_.notify_one();
    }
    return 0;
}

int Server::submit_many(const BatchItem* items, size_t n, uint64_t* tickets)
{
    if (!ok_) { set_error(-6, "server is not running"); return -6; }
    for (size_t i = 0; i < n; ++i) {        // validate and compile everything before queueing anything
        if (int rc = validate(items[i])) {
            set_error(rc, "request " + std::to_string(i) + ": " + last_error_string());
            return rc;
        }
    }
    const auto now = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(mu_);
    for (size_t i = 0; i < n; ++i) enqueue_locked(items[i], now, tickets[i]);
    cv_work_.notify_one();
    return 0;
}

int Server::wait_many(const uint64_t* tickets, size_t n, int timeout_ms)
{
    std::unique_lock<std::mutex> lk(mu_);
    for (size_t i = 0; i < n; ++i)
        if (recs_.find(tickets[i]) == recs_.end()) { set_error(-1, "unknown ticket"); return -1; }
    auto finished = [&](uint64_t t) { State s = recs_[t].state; return s == kDone || s == kFailed || s == kCancelled; };
    auto pred = [&] {
        for (size_t i = 0; i < n; ++i) if (!finished(tickets[i])) return false;
        return true;
    };
    if (timeout_ms < 0) cv_done_.wait(lk, pred);
    else if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) { set_error(-5, "wait timed out"); return -5; }
    for (size_t i = 0; i < n; ++i) {
        const State s = recs_[tickets[i]].state;
        if (s == kFailed) { set_error(-3, "request failed on the device"); return -3; }
        if (s == kCancelled) { set_error(-6, "request was cancelled"); return -6; }
    }
    return 0;
}

int Server::poll(uint64_t ticket)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = recs_.find(ticket);
    if (it == recs_.end()) return -1;
    switch (it->second.state) {
    case kDone: return 1;
    case kFailed: return -3;
    case kCancelled: return -6;
    default: return 0;
    }
}

int Server::wait(uint64_t ticket, int timeout_ms, float* minmax, float** dout)
{
    std::unique_lock<std::mutex> lk(mu_);
    auto it = recs_.find(ticket);
    if (it == recs_.end()) { set_error(-1, "unknown ticket"); return -1; }
    auto pred = [&] { State s = recs_[ticket].state; return s == kDone || s == kFailed || s == kCancelled; };
    if (timeout_ms < 0) cv_done_.wait(lk, pred);
    else if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) { set_error(-5, "wait timed out"); return -5; }
    Record& r = recs_[ticket];
    if (r.state == kFailed) { set_error(-3, "request failed on the device"); return -3; }
    if (r.state == kCancelled) { set_error(-6, "request was cancelled"); return -6; }
    if (minmax) { minmax[0] = r.minmax[0]; minmax[1] = r.minmax[1]; }
    if (dout) *dout = r.item.dout;
    return 0;
}

int Server::cancel(uint64_t ticket)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = recs_.find(ticket);
    if (it == recs_.end() || it->second.state != kQueued) return -6;
    queue_.erase(std::remove(queue_.begin(), queue_.end(), ticket), queue_.end());
    it->second.state = kCancelled;
    cv_done_.notify_all();
    return 0;
}

int Server::release(uint64_t ticket)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = recs_.find(ticket);
    if (it == recs_.end()) return -1;
    if (it->second.state == kQueued || it->second.state == kInflight) return -6;
    if (it->second.pooled) pool_.free(it->second.pool_off);
    node_unref(const_cast<Node*>(it->second.item.node));
    recs_.erase(it);
    return 0;
}

void Server::stats(ServerStats& s)
{
    std::lock_guard<std::mutex> lk(mu_);
    std::vector<double> v = lat_us_;
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) { return v.empty() ? 0.0 : v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
    s.submitted = submitted_;
    s.completed = completed_;
    s.failed = failed_;
    s.batches = batches_;
    s.points = points_;
    s.p50_us = pct(0.50);
    s.p99_us = pct(0.99);
    s.max_us = v.empty() ? 0.0 : v.back();
    double sum = 0;
    for (double x : v) sum += x;
    s.mean_us = v.empty() ? 0.0 : sum / v.size();
    s.pool_used = pool_.used();
    s.pool_capacity = pool_.capacity();
    s.queue_depth = (int)queue_.size();
    int inflight = 0;
    for (auto& kv : recs_) inflight += kv.second.state == kInflight;
    s.inflight = inflight;
    s.overlapped_batches = overlapped_;
    s.max_inflight_batches = max_inflight_;
    s.max_concurrent_batches = max_concurrent_;
}

void Server::reset_stats()
{
    std::lock_guard<std::mutex> lk(mu_);
    lat_us_.clear();
    submitted_ = completed_ = failed_ = batches_ = points_ = 0;
    spans_.clear();
    overlapped_ = 0;
    max_inflight_ = max_concurrent_ = 0;
}

// A retired batch's span of request completions on the device clock.  A batch that has
// completed a request by time t and completes another at t or later is executing at t, so
// two batches whose spans intersect were on the GPU together.
void Server::record_span(unsigned long long first, unsigned long long last)
{
    Span mine{first, last, false};
    for (Span& o : spans_) {
        if (o.first <= mine.last && mine.first <= o.last) {
            if (!o.counted) { o.counted = true; ++overlapped_; }
            if (!mine.counted) { mine.counted = true; ++overlapped_; }
        }
    }
    spans_.push_back(mine);
    if (spans_.size() > 64) spans_.pop_front();
    // most spans covering one moment: the maximum is reached at some span's start
    for (const Span& a : spans_) {
        int n = 0;
        for (const Span& b : spans_) n += b.first <= a.first && a.first <= b.last;
        max_concurrent_ = std::max(max_concurrent_, n);
    }
}

void Server::retire()
{
    bool any = false;
    const auto now = std::chrono::steady_clock::now();
    std::lock_guard<std::mutex> lk(mu_);
    for (auto& f : flights_) {
        if (!f.busy) continue;
        // Query the batch's event BEFORE sweeping the done flags: if the event has
        // completed, every flag the kernel raised is visible to this sweep, so a
        // request still unmarked afterwards really failed.  (Sweeping first would
        // race with a kernel that finishes between the sweep and the query.)
        const cudaError_t q = cudaEventQuery(f.done);
        bool all = true;
        for (uint64_t t : f.tickets) {
            Record& r = recs_[t];
            if (r.state != kInflight) continue;
            volatile Slot* sl = slots_ + r.slot;
            if (sl->done) {
                r.minmax[0] = sl->minmax[0];
                r.minmax[1] = sl->minmax[1];
                const unsigned long long td = sl->t_done;
                f.dev_first = std::min(f.dev_first, td);
                f.dev_last = std::max(f.dev_last, td);
                r.state = kDone;
                r.t_done = now;
                free_slots_.push_back(r.slot);
                lat_us_.push_back(std::chrono::duration<double, std::micro>(r.t_done - r.t_submit).count());
                ++completed_;
                points_ += (unsigned long long)std::max(0ll, r.item.args.total);
                any = true;
            } else {
                all = false;
            }
        }
        if (q == cudaSuccess) {
            if (!all) {                            // the batch finished without marking these requests
                for (uint64_t t : f.tickets) {
                    Record& r = recs_[t];
                    if (r.state == kInflight) { r.state = kFailed; free_slots_.push_back(r.slot); ++failed_; any = true; }
                }
                set_error(-3, "batch finished without completing every request");
            } else if (f.dev_first <= f.dev_last) {
                record_span(f.dev_first, f.dev_last);
            }
            f.busy = false;
            f.tickets.clear();
        } else if (q != cudaErrorNotReady) {
            for (uint64_t t : f.tickets) {
                Record& r = recs_[t];
                if (r.state == kInflight) { r.state = kFailed; free_slots_.push_back(r.slot); ++failed_; any = true; }
            }
            set_error(-3, std::string("batch failed: ") + cudaGetErrorString(q));
            f.busy = false;
            f.tickets.clear();
        }
    }
    if (any) cv_done_.notify_all();
}

bool Server::admit_and_launch(std::unique_lock<std::mutex>& lk)
{
    Flight* fl = nullptr;
    for (auto& f : flights_) if (!f.busy) { fl = &f; break; }
    if (!fl || queue_.empty()) return false;
    std::vector<BatchItem> items;
    std::vector<uint64_t> tickets;
    long long pts = 0;
    while (!queue_.empty() && (int)items.size() < cfg_.max_batch_requests && !free_slots_.empty()) {
        uint64_t t = queue_.front();
        Record& r = recs_[t];
        const long long n = std::max(0ll, r.item.args.total);
        if (!items.empty() && pts + n > cfg_.max_batch_points) break;
        if (!r.item.dout) {
            size_t off;
            if (!pool_.alloc((size_t)n * sizeof(float), off)) break;      // admission waits for memory
            r.pooled = true;
            r.pool_off = off;
            r.item.dout = reinterpret_cast<float*>(pool_.base() + off);
        }
        queue_.pop_front();
        r.slot = free_slots_.back();
        free_slots_.pop_back();
        slots_[r.slot].done = 0;
        r.item.host_done = &slots_dev_[r.slot].done;
        r.item.host_minmax = slots_dev_[r.slot].minmax;
        r.item.host_time = &slots_dev_[r.slot].t_done;
        r.item.dminmax = nullptr;
        r.state = kInflight;
        items.push_back(r.item);
        tickets.push_back(t);
        pts += n;
    }
    if (items.empty()) return false;
    fl->busy = true;
    fl->tickets = tickets;
    fl->dev_first = ~0ull;
    fl->dev_last = 0;
    ++batches_;
    int busy = 0;
    for (auto& f : flights_) busy += f.busy;
    max_inflight_ = std::max(max_inflight_, busy);
    lk.unlock();
    int rc = fl->runner->launch(items, fl->stream, nullptr, true);
    if (rc == 0) cudaEventRecord(fl->done, fl->stream);
    lk.lock();
    if (rc != 0) {
        for (uint64_t t : tickets) {
            Record& r = recs_[t];
            r.state = kFailed;
            free_slots_.push_back(r.slot);
            ++failed_;
        }
        fl->busy = false;
        fl->tickets.clear();
        cv_done_.notify_all();
    }
    return true;
}

void Server::loop()
{
    cudaSetDevice(device_);
    while (!stop_) {
        retire();
        std::unique_lock<std::mutex> lk(mu_);
        bool launched = admit_and_launch(lk);
        bool busy = false;
        for (auto& f : flights_) busy |= f.busy;
        if (!launched) {
            if (busy) {
                // Batches are on the GPU: poll their completion flags continuously.  A timed
                // sleep here would add the scheduler's wake-up delay (tens of microseconds)
                // to every request's latency.
                lk.unlock();
                std::this_thread::yield();
            } else {
                cv_work_.wait_for(lk, std::chrono::microseconds(cfg_.idle_wait_us > 0 ? cfg_.idle_wait_us : 50),
                                  [&] { return stop_.load() || !queue_.empty(); });
            }
        }
    }
    // drain: let in-flight batches finish, cancel what was never admitted
    for (auto& f : flights_) if (f.stream) cudaStreamSynchronize(f.stream);
    retire();
    std::lock_guard<std::mutex> lk(mu_);
    for (uint64_t t : queue_) recs_[t].state = kCancelled;
    queue_.clear();
    cv_done_.notify_all();
}

}  // namespace fn
