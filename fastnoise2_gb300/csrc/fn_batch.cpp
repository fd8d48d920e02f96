// fn_batch.cpp -- descriptor staging, graph capture and autotuning for the
// batched persistent launch (kernel in fn_kernels.cu).
#include "fn_batch.h"

#include "fn_jit.h"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace fn {

namespace {
size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }
}  // namespace

uint32_t tiles_for(long long total, uint32_t tile_points)
{
    if (total <= 0) return 1;                      // one empty tile still finalises min/max
    return (uint32_t)((total + tile_points - 1) / tile_points);
}

uint64_t batch_signature(const std::vector<BatchItem>& items, const std::vector<DeviceProgram>& progs)
{
    // multiset of (program, size class): independent of request order and of node addresses
    std::vector<uint64_t> keys;
    keys.reserve(items.size());
    for (size_t i = 0; i < items.size(); ++i) {
        int lg = 0;
        while ((1ll << lg) < items[i].args.total && lg < 62) ++lg;
        keys.push_back(progs[i].hash * 0x9E3779B97F4A7C15ull ^ ((uint64_t)items[i].args.src << 60) ^ ((uint64_t)lg << 48));
    }
    std::sort(keys.begin(), keys.end());
    return fnv1a64(keys.data(), keys.size() * sizeof(uint64_t));
}

BatchRunner::BatchRunner() {}

BatchRunner::~BatchRunner()
{
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    if (staged_) cudaEventDestroy(staged_);
    if (fork_) cudaEventDestroy(fork_);
    for (auto e : join_) cudaEventDestroy(e);
    for (auto a : aux_) cudaStreamDestroy(a);
    if (capture_stream_) cudaStreamDestroy(capture_stream_);
    if (d_buf_) cudaFree(d_buf_);
    if (h_buf_) cudaFreeHost(h_buf_);
}

bool BatchRunner::reserve(size_t n_req, size_t n_items)
{
    if (n_req <= cap_req_ && n_items <= cap_items_) return true;
    size_t req = std::max(n_req, std::max<size_t>(cap_req_ * 2, 64));
    size_t items = std::max(n_items, std::max<size_t>(cap_items_ * 2, 4096));
    size_t off_req = align_up(sizeof(BatchHeader), 256);
    size_t off_state = align_up(off_req + req * sizeof(BatchRequest), 256);
    size_t off_groups = align_up(off_state + req * sizeof(BatchState), 256);
    size_t off_items = align_up(off_groups + req * sizeof(BatchGroup), 256);
    size_t bytes = align_up(off_items + items * sizeof(uint2), 256);
    char* d = nullptr;
    char* h = nullptr;
    if (!cuda_ok(cudaMalloc(&d, bytes), "cudaMalloc(batch descriptors)")) return false;
    if (!cuda_ok(cudaMallocHost(&h, bytes), "cudaMallocHost(batch staging)")) { cudaFree(d); return false; }
    if (d_buf_) cudaFree(d_buf_);
    if (h_buf_) cudaFreeHost(h_buf_);
    d_buf_ = d; h_buf_ = h;
    cap_req_ = req; cap_items_ = items; cap_bytes_ = bytes;
    off_req_ = off_req; off_state_ = off_state; off_groups_ = off_groups; off_items_ = off_items;
    d_states_ = reinterpret_cast<BatchState*>(d_buf_ + off_state_);
    if (exec_) { cudaGraphExecDestroy(exec_); exec_ = nullptr; }   // kernel arguments changed: recapture
    if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
    return true;
}

bool BatchRunner::ensure_aux(size_t n)
{
    if (!fork_ && !cuda_ok(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming), "event")) return false;
    while (aux_.size() < n) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        if (!cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) return false;
        if (!cuda_ok(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event")) { cudaStreamDestroy(st); return false; }
        aux_.push_back(st);
        join_.push_back(ev);
    }
    return true;
}

cudaError_t BatchRunner::launch_group(size_t g, uint32_t smem, cudaStream_t stream)
{
    auto* hdr = reinterpret_cast<BatchHeader*>(d_buf_);
    auto* reqs = reinterpret_cast<BatchRequest*>(d_buf_ + off_req_);
    auto* items = reinterpret_cast<uint2*>(d_buf_ + off_items_);
    const Group& gr = groups_[g];
    if (!gr.jit) return launch_batch(hdr, reqs, d_states_, items, smem, gr.grid, 256, stream);
    BatchState* states = d_states_;
    BatchGroup* grp = reinterpret_cast<BatchGroup*>(d_buf_ + off_groups_) + g;
    void* params[] = {&hdr, &reqs, &states, &items, &grp};
    return cudaLaunchKernel((const void*)gr.jit, dim3((unsigned)gr.grid), dim3((unsigned)gr.threads), params, 0, stream);
}

// Several group kernels run concurrently: fork from `stream` onto the auxiliary
// streams (round robin), join back before anything later on `stream`.  Works the
// same inside a stream capture, where it becomes parallel graph branches.
bool BatchRunner::launch_groups(cudaStream_t stream, uint32_t smem)
{
    if (groups_.size() == 1) return cuda_ok(launch_group(0, smem, stream), "launch batch");
    const size_t na = std::min<size_t>(groups_.size(), 8);
    if (!ensure_aux(na)) return false;
    if (!cuda_ok(cudaEventRecord(fork_, stream), "fork")) return false;
    for (size_t a = 0; a < na; ++a)
        if (!cuda_ok(cudaStreamWaitEvent(aux_[a], fork_, 0), "fork wait")) return false;
    for (size_t g = 0; g < groups_.size(); ++g)
        if (!cuda_ok(launch_group(g, smem, aux_[g % na]), "launch batch group")) return false;
    for (size_t a = 0; a < na; ++a) {
        if (!cuda_ok(cudaEventRecord(join_[a], aux_[a]), "join")) return false;
        if (!cuda_ok(cudaStreamWaitEvent(stream, join_[a], 0), "join wait")) return false;
    }
    return true;
}

int BatchRunner::launch_graph(cudaStream_t stream, size_t bytes, uint32_t smem)
{
    // Recapture when the launch shape (kernels, grids, dynamic shared memory)
    // changed; otherwise only the upload node is updated -- the kernel arguments
    // are the fixed buffer addresses, the work lists travel in the upload.
    if (exec_ && (graph_groups_ != groups_ || graph_smem_ != smem)) {
        cudaGraphExecDestroy(exec_);
        exec_ = nullptr;
        if (graph_) { cudaGraphDestroy(graph_); graph_ = nullptr; }
    }
    if (!exec_) {
        graph_groups_ = groups_;
        graph_smem_ = smem;
        copy_node_ = nullptr;
        if (!capture_stream_ && !cuda_ok(cudaStreamCreateWithFlags(&capture_stream_, cudaStreamNonBlocking), "stream")) return -3;
        if (!cuda_ok(cudaStreamBeginCapture(capture_stream_, cudaStreamCaptureModeThreadLocal), "begin capture")) return -3;
        cudaMemcpyAsync(d_buf_, h_buf_, bytes, cudaMemcpyHostToDevice, capture_stream_);
        const bool queued = launch_groups(capture_stream_, smem);
        cudaGraph_t g = nullptr;
        const bool ended = cuda_ok(cudaStreamEndCapture(capture_stream_, &g), "end capture");
        if (!queued || !ended) { if (g) cudaGraphDestroy(g); return -3; }
        graph_ = g;
        if (!cuda_ok(cudaGraphInstantiate(&exec_, graph_, 0), "graph instantiate")) return -3;
        size_t n = 0;
        cudaGraphGetNodes(graph_, nullptr, &n);
        std::vector<cudaGraphNode_t> nodes(n);
        cudaGraphGetNodes(graph_, nodes.data(), &n);
        for (auto nd : nodes) {
            cudaGraphNodeType t;
            cudaGraphNodeGetType(nd, &t);
            if (t == cudaGraphNodeTypeMemcpy) copy_node_ = nd;
        }
        if (!copy_node_) { set_error(-3, "unexpected graph shape"); return -3; }
    } else {
        if (!cuda_ok(cudaGraphExecMemcpyNodeSetParams1D(exec_, copy_node_, d_buf_, h_buf_, bytes, cudaMemcpyHostToDevice), "graph memcpy update"))
            return -3;
    }
    return cuda_ok(cudaGraphLaunch(exec_, stream), "graph launch") ? 0 : -3;
}

int BatchRunner::launch(const std::vector<BatchItem>& items, cudaStream_t stream, const BatchTuning* tuning_in, bool use_graph)
{
    const size_t n = items.size();
    if (n == 0) return 0;
    std::vector<DeviceProgram> progs(n);
    uint32_t max_bytes = 16;
    points_ = 0;
    for (size_t i = 0; i < n; ++i) {
        if (!items[i].node || items[i].args.total < 0 || (items[i].args.total > 0 && !items[i].dout)) {
            set_error(-1, "batch request " + std::to_string(i) + ": invalid arguments");
            return -1;
        }
        if (!get_program(items[i].node, items[i].args.dim, progs[i])) return last_error();
        std::string err;
        if (!jit_ensure(progs[i].host, err)) { set_error(-2, "batch request " + std::to_string(i) + ": " + err); return -2; }
        max_bytes = std::max(max_bytes, progs[i].bytes);
        points_ += (uint64_t)std::max(0ll, items[i].args.total);
    }
    signature_ = batch_signature(items, progs);
    // Specialised batch kernels when every program of the batch has one: each tree's tuned
    // variant when it is built (a variant not built yet is queued for a background build and
    // variant 0 runs meanwhile), or the variant a tuning run forces.
    std::vector<BatchKernel> kernels(n);
    bool jit = true;
    for (size_t i = 0; jit && i < n; ++i) jit = items[i].args.total < (1ll << 32);   // 32-bit point indices
    {
        const int forced = tuning_in ? tuning_in->variant : -1;
        std::map<uint64_t, BatchKernel> chosen;
        for (size_t i = 0; jit && i < n; ++i) {
            auto it = chosen.find(progs[i].hash);
            if (it == chosen.end()) {
                BatchKernel bk;
                const int v = forced >= 0 ? forced : Autotuner::instance().tree_variant(progs[i].hash);
                bool ok = jit_batch_kernel(progs[i].hash, v, bk);
                if (!ok && !jit_is_specialised(progs[i].hash) && jit_try_cached(progs[i].host))   // an earlier process built it
                    ok = jit_batch_kernel(progs[i].hash, v, bk);
                if (!ok && v != 0) {
                    if (forced < 0) jit_request_batch_variants(progs[i].host);
                    ok = jit_batch_kernel(progs[i].hash, 0, bk);
                }
                if (!ok) { jit = false; break; }
                it = chosen.emplace(progs[i].hash, bk).first;
            }
            kernels[i] = it->second;
        }
    }
    if (!jit) {                                     // interpreter batch: count a use of each program
        std::vector<uint64_t> seen;
        for (size_t i = 0; i < n; ++i)
            if (std::find(seen.begin(), seen.end(), progs[i].hash) == seen.end()) {
                seen.push_back(progs[i].hash);
                jit_note_interpreted(progs[i].host);
            }
    }
    if (!jit)
        for (size_t i = 0; i < n; ++i)
            if (progs[i].host->needs_specialisation() && items[i].args.total > 0) {
                set_error(-2, "batch request " + std::to_string(i) + ": the tree needs specialised kernels, which this batch "
                              "cannot use (specialisation disabled or a request of 2^32 points or more)");
                return -2;
            }
    if (jit) signature_ = signature_ * 0x100000001B3ull + 0x4A17;   // tuned separately from the interpreter
    BatchTuning tuning;
    if (tuning_in) tuning = *tuning_in;
    else Autotuner::instance().lookup(signature_, tuning);
    const uint32_t tp = std::max<uint32_t>(256, tuning.tile_points);
    size_t n_items = 0;
    for (size_t i = 0; i < n; ++i) n_items += tiles_for(items[i].args.total, tp);
    if (n_items > 0xFFFFFFFFull) { set_error(-4, "batch too large"); return -4; }
    if (!reserve(n, n_items)) return -3;

    // Requests per group: all of them for the interpreter, one group per
    // distinct specialised kernel (first-appearance order) otherwise.
    std::vector<std::vector<uint32_t>> members;
    std::vector<BatchKernel> gkernel;
    if (jit) {
        std::map<cudaKernel_t, size_t> index;
        for (size_t i = 0; i < n; ++i) {
            auto it = index.find(kernels[i].kernel);
            if (it == index.end()) {
                it = index.emplace(kernels[i].kernel, members.size()).first;
                members.emplace_back();
                gkernel.push_back(kernels[i]);
            }
            members[it->second].push_back((uint32_t)i);
        }
    } else {
        members.emplace_back();
        gkernel.push_back(BatchKernel{nullptr, 256});          // the interpreter's batch kernel: 256 threads
        for (size_t i = 0; i < n; ++i) members[0].push_back((uint32_t)i);
    }

    // The staging buffer is reused: the previous launch's upload must have been consumed.
    if (!staged_ && !cuda_ok(cudaEventCreateWithFlags(&staged_, cudaEventDisableTiming), "event")) return -3;
    cudaEventSynchronize(staged_);

    auto* hdr = reinterpret_cast<BatchHeader*>(h_buf_);
    auto* reqs = reinterpret_cast<BatchRequest*>(h_buf_ + off_req_);
    auto* states = reinterpret_cast<BatchState*>(h_buf_ + off_state_);
    auto* grps = reinterpret_cast<BatchGroup*>(h_buf_ + off_groups_);
    auto* its = reinterpret_cast<uint2*>(h_buf_ + off_items_);
    std::memset(hdr, 0, sizeof(BatchHeader));
    hdr->n_req = (unsigned)n;
    hdr->n_items = (unsigned)n_items;
    hdr->tile_points = tp;
    hdr->max_prog_bytes = max_bytes;
    last_minmax_.resize(n);
    for (size_t i = 0; i < n; ++i) {
        BatchRequest& r = reqs[i];
        std::memset(&r, 0, sizeof r);
        r.args = items[i].args;
        r.prog = progs[i].dptr;
        r.jit_slot = -1;
        r.prog_bytes = progs[i].bytes;
        r.out = items[i].dout;
        r.minmax = items[i].dminmax;
        r.host_minmax = items[i].host_minmax;
        r.host_done = items[i].host_done;
        r.host_time = items[i].host_time;
        r.n_tiles = tiles_for(items[i].args.total, tp);
        states[i].mn_enc = 0xFFFFFFFFu;
        states[i].mx_enc = 0u;
        states[i].tiles_done = 0u;
        states[i].pad = 0u;
        last_minmax_[i] = items[i].dminmax;
    }
    const int sms = num_sms();
    groups_.assign(members.size(), Group());
    size_t k = 0;
    int total_grid = 0;
    for (size_t g = 0; g < members.size(); ++g) {
        Group& gr = groups_[g];
        gr.jit = gkernel[g].kernel;
        gr.threads = gkernel[g].threads;
        gr.item_begin = (uint32_t)k;
        for (uint32_t i : members[g])
            for (uint32_t t = 0; t < reqs[i].n_tiles; ++t) its[k++] = make_uint2(i, t);
        gr.item_end = (uint32_t)k;
        grps[g].item_begin = gr.item_begin;
        grps[g].item_end = gr.item_end;
        grps[g].head = 0;
        grps[g].pad = 0;
        int occ = tuning.ctas_per_sm;
        if (occ <= 0 && gr.jit) {
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void*)gr.jit, gr.threads, 0) != cudaSuccess || occ < 1) occ = 1;
        } else if (occ <= 0) {
            occ = batch_occupancy(256, max_bytes);
        }
        long long grid = (long long)sms * occ;
        const long long group_items = (long long)(gr.item_end - gr.item_begin);
        if (grid > group_items) grid = group_items;
        if (grid < 1) grid = 1;
        gr.grid = (int)grid;
        total_grid += gr.grid;
    }
    const size_t bytes = off_items_ + n_items * sizeof(uint2);
    const uint32_t smem = jit ? 0 : max_bytes;
    // A graph pays off for a launch shape that repeats (the same batch every frame); batches
    // whose shape keeps changing (a server's admissions) would pay a capture each time, so a
    // new shape is captured only when it comes twice in a row and runs as plain launches until then.
    const bool same_as_graph = exec_ && graph_groups_ == groups_ && graph_smem_ == smem;
    const bool repeated = last_groups_ == groups_ && last_smem_ == smem;
    last_groups_ = groups_;
    last_smem_ = smem;
    int rc;
    if (use_graph && (same_as_graph || repeated)) {
        rc = launch_graph(stream, bytes, smem);
    } else {
        rc = cuda_ok(cudaMemcpyAsync(d_buf_, h_buf_, bytes, cudaMemcpyHostToDevice, stream), "upload batch") &&
                     launch_groups(stream, smem)
                 ? 0
                 : -3;
    }
    if (rc == 0) {
        cudaEventRecord(staged_, stream);
        items_ = n_items;
        upload_bytes_ = bytes;
        tile_points_ = tp;
        grid_ = total_grid;
        specialised_ = jit;
    }
    return rc;
}

// ------------------------------------------------------------------ autotuner

Autotuner& Autotuner::instance()
{
    static Autotuner a;
    return a;
}

bool Autotuner::lookup(uint64_t sig, BatchTuning& out)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = table_.find(sig);
    if (it == table_.end()) return false;
    out = it->second.first;
    return true;
}

void Autotuner::store(uint64_t sig, const BatchTuning& t, double ms)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = table_.find(sig);
    if (it == table_.end() || ms < it->second.second) table_[sig] = {t, ms};
}

std::vector<BatchTuning> Autotuner::candidates() const
{
    std::vector<BatchTuning> c;
    for (uint32_t tp : {1024u, 2048u, 4096u, 8192u})
        for (int ctas : {0, 1}) c.push_back(BatchTuning{tp, ctas, -1});
    return c;
}

int Autotuner::tree_variant(uint64_t program_hash)
{
    std::lock_guard<std::mutex> lk(mu_);
    auto it = trees_.find(program_hash);
    return it == trees_.end() ? 0 : it->second.first;
}

void Autotuner::store_tree(uint64_t program_hash, int variant, double ms)
{
    std::lock_guard<std::mutex> lk(mu_);
    trees_[program_hash] = {variant, ms};
}

// Text format, one entry per line:
//   <signature hex> <tile points> <CTAs per SM> <ms>                         a batch signature
//   tree <program hash hex> <variant> <threads> <blocks per SM> <points> <ms>  a tree's batch kernel
bool Autotuner::load(const std::string& path)
{
    std::ifstream f(path);
    if (!f) return false;
    std::lock_guard<std::mutex> lk(mu_);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream in(line);
        std::string first;
        if (!(in >> first)) continue;
        if (first == "tree") {
            unsigned long long hash;
            int variant, threads, blocks, points;
            double ms;
            if (in >> std::hex >> hash >> std::dec >> variant >> threads >> blocks >> points >> ms && variant >= 0 &&
                (size_t)variant < batch_variants().size())
                trees_[hash] = {variant, ms};
        } else {
            unsigned long long sig = std::strtoull(first.c_str(), nullptr, 16);
            unsigned tp;
            int ctas;
            double ms;
            if (in >> tp >> ctas >> ms) table_[sig] = {BatchTuning{tp, ctas, -1}, ms};
        }
    }
    return true;
}

bool Autotuner::save(const std::string& path) const
{
    std::ofstream f(path);
    if (!f) return false;
    for (const auto& kv : table_)
        f << std::hex << kv.first << std::dec << ' ' << kv.second.first.tile_points << ' ' << kv.second.first.ctas_per_sm << ' '
          << kv.second.second << '\n';
    for (const auto& kv : trees_) {
        const BatchVariant& v = batch_variants()[(size_t)kv.second.first];
        f << "tree " << std::hex << kv.first << std::dec << ' ' << kv.second.first << ' ' << v.threads << ' ' << v.min_blocks << ' '
          << v.points << ' ' << kv.second.second << '\n';
    }
    return true;
}

}  // namespace fn
