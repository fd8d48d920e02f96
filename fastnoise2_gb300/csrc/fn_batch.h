// fn_batch.h -- many generation requests in one persistent launch.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fn_kernels.cuh"
#include "fn_runtime.h"

namespace fn {

struct BatchItem {
    const Node* node = nullptr;
    PointArgs args{};
    float* dout = nullptr;
    float* dminmax = nullptr;          // device float[2] or null
    float* host_minmax = nullptr;      // mapped pinned float[2] or null
    unsigned int* host_done = nullptr; // mapped pinned completion flag or null
    unsigned long long* host_time = nullptr;  // mapped pinned: device clock (ns) at completion, or null
};

struct BatchTuning {
    uint32_t tile_points = 2048;
    int ctas_per_sm = 0;               // 0 = occupancy limit
    int variant = -1;                  // specialised kernel variant for every tree; -1 = each tree's tuned choice
};

// Owns the device/pinned descriptor buffers and a captured graph; not thread safe
// (one runner per host thread or per server stream).
class BatchRunner {
public:
    BatchRunner();
    ~BatchRunner();
    BatchRunner(const BatchRunner&) = delete;
    BatchRunner& operator=(const BatchRunner&) = delete;

    // Resolve programs, build descriptors and queue one launch on `stream`.
    // Returns FN_OK or a negative status (set_error has the message).
    // `tuning` null = the autotuner's choice for this batch signature, else defaults.
    int launch(const std::vector<BatchItem>& items, cudaStream_t stream, const BatchTuning* tuning, bool use_graph);

    // Device copy of the last launch's per-request state (for min/max read-back).
    BatchState* device_states() const { return d_states_; }
    const std::vector<float*>& last_device_minmax() const { return last_minmax_; }
    uint64_t last_signature() const { return signature_; }
    uint64_t last_points() const { return points_; }
    // Shape of the last launch: work items, bytes uploaded, tile size, CTAs, kernel kind.
    uint64_t last_items() const { return items_; }
    uint64_t last_upload_bytes() const { return upload_bytes_; }
    uint32_t last_tile_points() const { return tile_points_; }
    int last_grid() const { return grid_; }
    bool last_specialised() const { return specialised_; }
    int last_kernels() const { return (int)groups_.size(); }

private:
    // One kernel launch of a batch: the interpreter's batch kernel over all items
    // (jit null), or one tree's specialised batch kernel over that tree's items.
    struct Group {
        cudaKernel_t jit = nullptr;
        int threads = 256;
        uint32_t item_begin = 0, item_end = 0;
        int grid = 1;
        bool operator==(const Group& o) const { return jit == o.jit && grid == o.grid && threads == o.threads; }
    };
    bool reserve(size_t n_req, size_t n_items);
    int launch_graph(cudaStream_t stream, size_t bytes, uint32_t smem);
    // Queue the upload-free part: every group's kernel, forked over the auxiliary
    // streams and joined back into `stream` when there is more than one.
    bool launch_groups(cudaStream_t stream, uint32_t smem);
    cudaError_t launch_group(size_t g, uint32_t smem, cudaStream_t stream);
    bool ensure_aux(size_t n);

    char* d_buf_ = nullptr;            // device: header | reqs | states | groups | items
    char* h_buf_ = nullptr;            // pinned staging with the same layout
    size_t cap_req_ = 0, cap_items_ = 0, cap_bytes_ = 0;
    size_t off_req_ = 0, off_state_ = 0, off_groups_ = 0, off_items_ = 0;
    BatchState* d_states_ = nullptr;
    std::vector<Group> groups_;
    std::vector<cudaStream_t> aux_;     // fork/join streams for concurrent group kernels
    std::vector<cudaEvent_t> join_;
    cudaEvent_t fork_ = nullptr;
    cudaStream_t capture_stream_ = nullptr;
    cudaEvent_t staged_ = nullptr;      // recorded after each upload: guards reuse of h_buf_
    cudaGraph_t graph_ = nullptr;
    cudaGraphExec_t exec_ = nullptr;
    cudaGraphNode_t copy_node_ = nullptr;
    std::vector<Group> graph_groups_;   // launch shape the graph was captured with
    uint32_t graph_smem_ = 0;
    std::vector<Group> last_groups_;    // shape of the previous launch (a graph is captured for a repeated shape)
    uint32_t last_smem_ = 0;
    std::vector<float*> last_minmax_;
    uint64_t signature_ = 0;
    uint64_t points_ = 0;
    uint64_t items_ = 0, upload_bytes_ = 0;
    uint32_t tile_points_ = 0;
    int grid_ = 0;
    bool specialised_ = false;
};

// Tuning cache: per batch signature (program hashes and size classes) the tile size and
// CTAs per SM; per tree (program hash, which includes the dimensionality) the variant of its
// specialised batch kernel.  Saved and loaded as text.
class Autotuner {
public:
    static Autotuner& instance();
    bool lookup(uint64_t signature, BatchTuning& out);
    void store(uint64_t signature, const BatchTuning& t, double ms);
    std::vector<BatchTuning> candidates() const;
    int tree_variant(uint64_t program_hash);                 // 0 when the tree has not been tuned
    void store_tree(uint64_t program_hash, int variant, double ms);
    bool load(const std::string& path);
    bool save(const std::string& path) const;

private:
    std::mutex mu_;
    std::map<uint64_t, std::pair<BatchTuning, double>> table_;
    std::map<uint64_t, std::pair<int, double>> trees_;
};

uint64_t batch_signature(const std::vector<BatchItem>& items, const std::vector<DeviceProgram>& progs);
uint32_t tiles_for(long long total, uint32_t tile_points);

}  // namespace fn
