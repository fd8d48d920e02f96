// fn_server.h -- continuous-batching request server.
//
// The reference has no server; its closest analogue is the Node Editor's CPU
// worker pool that generates one chunk per thread (tools/NodeEditor/
// MeshNoisePreview.cpp:88-95, :397-414).  Here one loop thread:
//   * admits queued requests while the device pool can hold their outputs and
//     an in-flight slot is free (admission defers, never fails, unless a request
//     can never fit);
//   * launches admitted requests as one persistent batch on a free stream,
//     while earlier batches are still running on the others;
//   * retires each request as soon as the kernel marks its last tile done
//     (a flag in mapped pinned memory), records its latency and frees its slot.
#pragma once
#include <cuda_runtime.h>

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

#include "fn_batch.h"

namespace fn {

struct ServerConfig {
    size_t pool_bytes = size_t(1) << 30;
    int streams = 3;                  // batches in flight at once
    int max_batch_requests = 1024;
    long long max_batch_points = 64ll << 20;
    int idle_wait_us = 50;
};

// First-fit allocator over one device reservation (256-byte granules).
class DevicePool {
public:
    bool init(size_t bytes);
    ~DevicePool();
    bool alloc(size_t bytes, size_t& offset);
    void free(size_t offset);
    char* base() const { return base_; }
    size_t capacity() const { return cap_; }
    size_t used() const { return used_; }

private:
    char* base_ = nullptr;
    size_t cap_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;        // offset -> size
    std::unordered_map<size_t, size_t> live_;
};

struct ServerStats {
    unsigned long long submitted, completed, failed, batches;
    unsigned long long points;
    double p50_us, p99_us, max_us, mean_us;
    size_t pool_used, pool_capacity;
    int queue_depth, inflight;
    // Batches whose requests completed, on the device clock, within another batch's span of
    // completions: both batches were executing on the GPU at the same moment.
    unsigned long long overlapped_batches;
    int max_inflight_batches;         // most batches launched and not yet retired at once
    int max_concurrent_batches;       // most batches executing on the GPU at one moment (device clock)
};

class Server {
public:
    explicit Server(const ServerConfig& cfg);
    ~Server();
    bool ok() const { return ok_; }

    int submit(const BatchItem& item, uint64_t& ticket);      // item.dout null => pool-allocated output
    // All-or-nothing submission of n items under one lock (tickets[i] for items[i]).
    int submit_many(const BatchItem* items, size_t n, uint64_t* tickets);
    // Open-loop submission: item k is submitted when the steady clock reaches start + arrival_us[k]
    // (the calling thread waits until then), and its latency counts from that arrival time, so
    // a submitter falling behind the schedule shows up in the latency.
    int submit_paced(const BatchItem* items, size_t n, const double* arrival_us, uint64_t* tickets);
    // Wait until every ticket is finished (done, failed or cancelled); FN_ERR_TIMEOUT if
    // timeout_ms >= 0 runs out first.  Returns 0, or the first failure's status.
    int wait_many(const uint64_t* tickets, size_t n, int timeout_ms);
    int poll(uint64_t ticket);                                   // 1 done, 0 pending, < 0 error
    int wait(uint64_t ticket, int timeout_ms, float* minmax, float** dout);
    int cancel(uint64_t ticket);                                 // only before admission
    int release(uint64_t ticket);
    void stats(ServerStats& s);
    void reset_stats();

private:
    enum State { kQueued, kInflight, kDone, kFailed, kCancelled };
    struct Record {
        State state = kQueued;
        BatchItem item;
        bool pooled = false;
        size_t pool_off = 0;
        int slot = -1;
        float minmax[2] = {0, 0};
        std::chrono::steady_clock::time_point t_submit, t_done;
    };
    struct Flight {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        std::unique_ptr<BatchRunner> runner;
        std::vector<uint64_t> tickets;
        bool busy = false;
        unsigned long long dev_first = ~0ull, dev_last = 0;   // device clock of the first and last completion
    };
    struct Slot {                      // mapped pinned, written by the kernel that completes the request
        unsigned int done;
        unsigned int pad;
        float minmax[2];
        unsigned long long t_done;     // device clock (ns)
    };
    struct Span {
        unsigned long long first, last;
        bool counted;
    };

    int enqueue_locked(const BatchItem& item, std::chrono::steady_clock::time_point t_submit, uint64_t& ticket);
    int validate(const BatchItem& item);
    void record_span(unsigned long long first, unsigned long long last);

    void loop();
    bool admit_and_launch(std::unique_lock<std::mutex>& lk);
    void retire();

    ServerConfig cfg_;
    bool ok_ = false;
    DevicePool pool_;
    Slot* slots_ = nullptr;            // mapped pinned
    Slot* slots_dev_ = nullptr;
    int n_slots_ = 0;
    std::vector<int> free_slots_;
    std::vector<Flight> flights_;

    std::mutex mu_;
    std::condition_variable cv_work_, cv_done_;
    std::deque<uint64_t> queue_;
    std::unordered_map<uint64_t, Record> recs_;
    std::atomic<bool> stop_{false};
    uint64_t next_ticket_ = 1;
    std::thread thread_;
    int device_ = 0;

    // statistics
    std::vector<double> lat_us_;
    unsigned long long submitted_ = 0, completed_ = 0, failed_ = 0, batches_ = 0, points_ = 0;
    std::deque<Span> spans_;           // completion spans of the most recent batches
    unsigned long long overlapped_ = 0;
    int max_inflight_ = 0, max_concurrent_ = 0;
};

}  // namespace fn
