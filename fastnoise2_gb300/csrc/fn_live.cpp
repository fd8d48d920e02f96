// fn_live.cpp -- live trees: a tree that follows the Node Editor's channel (fnLiveTree* in
// include/FastNoise/FastNoise_C.h).
//
// The reference's editor publishes the selected tree as an encoded string on its shared-memory
// channel (tools/NodeEditorIpc/NodeEditorIpc_C.cpp:182-281; sent from
// tools/NodeEditor/FastNoiseNodeEditor.cpp:1581); a consumer polls it and builds a new
// generator.  Here an update decodes the string, compiles the tree for every dimensionality
// the caller generates with (device program upload, and NVRTC specialisation when enabled),
// and only then swaps it in under a lock, so a generation or serving thread that acquires the
// tree always gets a fully built one.  The swapped-out tree is released by reference count:
// requests already submitted with it (the server holds a reference per request) finish with it.
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/FastNoise/FastNoise_C.h"
#include "../../include/FastNoise/NodeEditorIpc_C.h"
#include "fn_jit.h"
#include "fn_node.h"
#include "fn_runtime.h"

using namespace fn;

namespace {

struct LiveTree {
    void* ipc = nullptr;                  // not owned
    std::vector<int> dims;
    std::mutex mu;                        // current tree and info
    Node* current = nullptr;
    fnLiveTreeInfo info{};
    std::mutex update_mu;                 // one update at a time
    std::vector<char> buf = std::vector<char>(64 * 1024);
    std::thread poller;
    int device = 0;                       // the creating thread's device, used by the poller
    std::mutex stop_mu;
    std::condition_variable stop_cv;
    bool stop = false;
};

// Compile `node` for every dimensionality (and specialise it when enabled); FN_OK or FN_ERR_*.
int prepare(Node* node, const std::vector<int>& dims)
{
    for (int d : dims) {
        DeviceProgram dp;
        if (!get_program(node, d, dp)) return last_error() ? last_error() : FN_ERR_COMPILE;
    }
    if (jit_enabled()) {
        std::vector<const void*> nodes(dims.size(), node);
        const int rc = fnJitCompile(nodes.data(), dims.data(), (int)dims.size());
        if (rc != FN_OK) return rc;
    }
    return FN_OK;
}

void reject(LiveTree* lt, int code, const std::string& why)
{
    std::lock_guard<std::mutex> lk(lt->mu);
    lt->info.rejected++;
    lt->info.lastStatus = code;
    std::strncpy(lt->info.lastError, why.c_str(), sizeof(lt->info.lastError) - 1);
    lt->info.lastError[sizeof(lt->info.lastError) - 1] = '\0';
}

// Decode, build and swap in one encoded tree: 1 = now current, FN_ERR_* = rejected.
int install(LiveTree* lt, const char* encoded)
{
    Node* n = decode_tree(encoded);
    if (!n) {
        reject(lt, FN_ERR_ARG, "the encoded node tree does not decode");
        set_error(FN_ERR_ARG, "live tree: the encoded node tree does not decode");
        return FN_ERR_ARG;
    }
    const int rc = prepare(n, lt->dims);
    if (rc != FN_OK) {
        const std::string why = last_error_string();
        node_unref(n);
        reject(lt, rc, why);
        set_error(rc, "live tree: " + why);
        return rc;
    }
    Node* old = nullptr;
    {
        std::lock_guard<std::mutex> lk(lt->mu);
        old = lt->current;
        lt->current = n;
        lt->info.version++;
    }
    if (old) node_unref(old);
    return 1;
}

int update(LiveTree* lt)
{
    std::lock_guard<std::mutex> lk(lt->update_mu);
    if (!lt->ipc) return 0;
    int newest = 0;
    // drain the channel: only a selected-node message is for us (import requests go to the editor)
    for (int k = 0; k < 64; ++k) {
        const int type = fnEditorIpcPollMessage(lt->ipc, lt->buf.data(), (int)lt->buf.size());
        if (type == FASTNOISE_EDITORIPC_MSG_NONE) break;
        if (type != FASTNOISE_EDITORIPC_MSG_SELECTED_NODE) continue;
        newest = install(lt, lt->buf.data());
    }
    return newest;
}

void poll_loop(LiveTree* lt, int period_ms)
{
    cudaSetDevice(lt->device);
    std::unique_lock<std::mutex> lk(lt->stop_mu);
    while (!lt->stop) {
        lk.unlock();
        update(lt);
        lk.lock();
        lt->stop_cv.wait_for(lk, std::chrono::milliseconds(period_ms), [lt] { return lt->stop; });
    }
}

}  // namespace

extern "C" {

void* fnLiveTreeCreate(void* ipc, const char* initialEncodedTree, const int* dimensions, int count, int pollMs)
{
    clear_error();
    if (!dimensions || count < 1 || count > 3 || pollMs < 0) {
        set_error(FN_ERR_ARG, "invalid arguments");
        return nullptr;
    }
    LiveTree* lt = new LiveTree();
    lt->ipc = ipc;
    cudaGetDevice(&lt->device);
    for (int i = 0; i < count; ++i) {
        if (dimensions[i] < 2 || dimensions[i] > 4) {
            delete lt;
            set_error(FN_ERR_ARG, "dimensions must be 2, 3 or 4");
            return nullptr;
        }
        lt->dims.push_back(dimensions[i]);
    }
    if (initialEncodedTree && initialEncodedTree[0] && install(lt, initialEncodedTree) != 1) {
        delete lt;                          // the reason is in fnGetLastErrorString
        return nullptr;
    }
    if (pollMs > 0 && ipc) lt->poller = std::thread(poll_loop, lt, pollMs);
    return lt;
}

int fnLiveTreeUpdate(void* live)
{
    clear_error();
    if (!live) {
        set_error(FN_ERR_ARG, "null live tree");
        return FN_ERR_ARG;
    }
    return update(static_cast<LiveTree*>(live));
}

void* fnLiveTreeAcquire(void* live, unsigned long long* version)
{
    if (!live) return nullptr;
    LiveTree* lt = static_cast<LiveTree*>(live);
    std::lock_guard<std::mutex> lk(lt->mu);
    if (version) *version = lt->info.version;
    if (lt->current) node_ref(lt->current);
    return lt->current;
}

int fnLiveTreeGetInfo(void* live, fnLiveTreeInfo* info)
{
    if (!live || !info) return FN_ERR_ARG;
    LiveTree* lt = static_cast<LiveTree*>(live);
    std::lock_guard<std::mutex> lk(lt->mu);
    *info = lt->info;
    return FN_OK;
}

void fnLiveTreeDelete(void* live)
{
    if (!live) return;
    LiveTree* lt = static_cast<LiveTree*>(live);
    if (lt->poller.joinable()) {
        {
            std::lock_guard<std::mutex> lk(lt->stop_mu);
            lt->stop = true;
        }
        lt->stop_cv.notify_all();
        lt->poller.join();
    }
    if (lt->current) node_unref(lt->current);
    delete lt;
}

}  // extern "C"
