// fn_ipc.cpp -- the Node Editor's shared-memory channel (include/FastNoise/NodeEditorIpc_C.h).
//
// Same object name, size and message layout as the reference's NodeEditorIpc library
// (tools/NodeEditorIpc/NodeEditorIpc_C.cpp:32-33, 130-281), so that this library and a running
// FastNoise2 Node Editor exchange trees:
//   byte 0   message counter, incremented by the sender after the rest is written
//   byte 1   message type (selected node / import request)
//   byte 2.. NUL-terminated encoded node tree
// A context remembers the last counter it has seen; a sender marks its own message as seen.
// The counter is read and written with acquire / release atomics so that a poller that sees a
// new counter also sees the payload written before it.
#include <dlfcn.h>
#include <fcntl.h>
#include <spawn.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/FastNoise/NodeEditorIpc_C.h"

extern char** environ;

namespace {

constexpr const char* kChannelName = "/FastNoise2NodeEditor";
constexpr size_t kChannelBytes = 64 * 1024;
constexpr size_t kHeaderBytes = 2;

struct EditorChannel {
    unsigned char* mem = nullptr;
    unsigned char seen = 0;            // counter value of the last message handled or sent
};

unsigned char load_counter(const unsigned char* mem) { return __atomic_load_n(mem, __ATOMIC_ACQUIRE); }
void store_counter(unsigned char* mem, unsigned char v) { __atomic_store_n(mem, v, __ATOMIC_RELEASE); }

bool send(void* ipc, unsigned char type, const char* tree)
{
    EditorChannel* ch = static_cast<EditorChannel*>(ipc);
    if (!ch || !ch->mem || !tree) return false;
    const size_t n = std::strlen(tree);
    if (n + kHeaderBytes + 1 >= kChannelBytes) return false;
    std::memcpy(ch->mem + kHeaderBytes, tree, n + 1);
    ch->mem[1] = type;
    const unsigned char next = (unsigned char)(load_counter(ch->mem) + 1u);
    store_counter(ch->mem, next);
    ch->seen = next;
    return true;
}

std::mutex g_path_mu;
std::string g_editor_path;

bool executable(const std::string& p) { return !p.empty() && access(p.c_str(), X_OK) == 0; }

std::string find_editor()
{
    {
        std::lock_guard<std::mutex> lk(g_path_mu);
        if (!g_editor_path.empty()) return g_editor_path;
    }
    Dl_info info;
    if (dladdr(reinterpret_cast<void*>(&fnEditorIpcSetup), &info) && info.dli_fname) {
        std::string dir(info.dli_fname);
        const size_t slash = dir.find_last_of('/');
        dir = slash == std::string::npos ? std::string(".") : dir.substr(0, slash);
        for (const char* rel : {"/NodeEditor", "/../bin/NodeEditor"})
            if (executable(dir + rel)) return dir + rel;
    }
    for (const char* p : {"./NodeEditor", "../bin/NodeEditor", "./bin/NodeEditor"})
        if (executable(p)) return p;
    return std::string();
}

}  // namespace

extern "C" {

void* fnEditorIpcSetup(bool readPrevious)
{
    const int fd = shm_open(kChannelName, O_CREAT | O_RDWR, 0666);
    if (fd < 0) return nullptr;
    struct stat st;
    if (fstat(fd, &st) != 0 || (size_t)st.st_size < kChannelBytes) {
        if (ftruncate(fd, kChannelBytes) != 0 && errno != EINVAL) {
            close(fd);
            return nullptr;
        }
    }
    void* mem = mmap(nullptr, kChannelBytes, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
    close(fd);
    if (mem == MAP_FAILED) return nullptr;
    EditorChannel* ch = new EditorChannel();
    ch->mem = static_cast<unsigned char*>(mem);
    const unsigned char counter = load_counter(ch->mem);
    // readPrevious: treat a waiting selected-node message as unseen
    ch->seen = (readPrevious && ch->mem[1] == FASTNOISE_EDITORIPC_MSG_SELECTED_NODE) ? (unsigned char)(counter - 1u) : counter;
    return ch;
}

void fnEditorIpcRelease(void* ipc)
{
    EditorChannel* ch = static_cast<EditorChannel*>(ipc);
    if (!ch) return;
    if (ch->mem) munmap(ch->mem, kChannelBytes);
    shm_unlink(kChannelName);
    delete ch;
}

bool fnEditorIpcSendSelectedNode(void* ipc, const char* encodedNodeTree)
{
    return send(ipc, FASTNOISE_EDITORIPC_MSG_SELECTED_NODE, encodedNodeTree);
}

bool fnEditorIpcSendImportRequest(void* ipc, const char* encodedNodeTree)
{
    return send(ipc, FASTNOISE_EDITORIPC_MSG_IMPORT_REQUEST, encodedNodeTree);
}

int fnEditorIpcPollMessage(void* ipc, char* outBuffer, int bufferSize)
{
    EditorChannel* ch = static_cast<EditorChannel*>(ipc);
    if (!ch || !ch->mem) return FASTNOISE_EDITORIPC_MSG_IPC_NOT_INITIALISED;
    const unsigned char counter = load_counter(ch->mem);
    if (counter == ch->seen) return FASTNOISE_EDITORIPC_MSG_NONE;
    const int type = ch->mem[1];
    if (type != FASTNOISE_EDITORIPC_MSG_SELECTED_NODE && type != FASTNOISE_EDITORIPC_MSG_IMPORT_REQUEST) {
        ch->seen = counter;                          // not a message for anyone: skip it
        return FASTNOISE_EDITORIPC_MSG_NONE;
    }
    if (!outBuffer || bufferSize <= 0) return FASTNOISE_EDITORIPC_MSG_BUFFER_TOO_SMALL;
    ch->seen = counter;                              // consumed, as in the reference, even if it does not fit
    const char* tree = reinterpret_cast<const char*>(ch->mem + kHeaderBytes);
    const size_t n = strnlen(tree, kChannelBytes - kHeaderBytes - 1);
    if (n + 1 > (size_t)bufferSize) return FASTNOISE_EDITORIPC_MSG_BUFFER_TOO_SMALL;
    std::memcpy(outBuffer, tree, n);
    outBuffer[n] = '\0';
    return type;
}

void fnEditorIpcSetNodeEditorPath(const char* path)
{
    std::lock_guard<std::mutex> lk(g_path_mu);
    g_editor_path = path ? path : "";
}

bool fnEditorIpcStartNodeEditor(const char* encodedNodeTree, bool detached, bool childProcess)
{
    const std::string exe = find_editor();
    if (exe.empty()) return false;
    std::vector<std::string> args{exe};
    if (detached) args.push_back("--detached");
    if (encodedNodeTree && encodedNodeTree[0]) {
        args.push_back("--import-ent");
        args.push_back(encodedNodeTree);
    }
    std::vector<char*> argv;
    for (std::string& a : args) argv.push_back(&a[0]);
    argv.push_back(nullptr);
    posix_spawnattr_t attr;
    if (posix_spawnattr_init(&attr) != 0) return false;
#ifdef POSIX_SPAWN_SETSID
    if (!childProcess) posix_spawnattr_setflags(&attr, POSIX_SPAWN_SETSID);   // outlives this process's session
#endif
    pid_t pid = 0;
    const int rc = posix_spawn(&pid, exe.c_str(), nullptr, &attr, argv.data(), environ);
    posix_spawnattr_destroy(&attr);
    return rc == 0;
}

}  // extern "C"
