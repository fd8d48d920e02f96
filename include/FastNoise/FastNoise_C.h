/*
 * FastNoise_C.h -- C-ABI of the GB300 FastNoise2 backend (libfastnoise_gb300.so).
 *
 * Drop-in for FastNoise2's own C-ABI (reference include/FastNoise/FastNoise_C.h,
 * implemented in src/FastNoise/FastNoise_C.cpp).  Every function in the first
 * part keeps the reference's name, argument meaning and error behaviour; the
 * citation beside each one is the reference declaration it replaces.  Node
 * handles are opaque, reference counted, and may be shared between threads for
 * generation (README.md:39-40 of the reference).  Node trees are evaluated on
 * the current CUDA device; output arrays in this part are HOST memory.
 *
 * The second part adds entry points that the reference does not have: device
 * pointer variants (output stays in GPU memory), tree serialisation, batched
 * generation and a request server.  They return an int status (0 = ok,
 * negative = error, text via fnGetLastErrorString()).
 *
 * Where the reference would compute on the CPU, this library never does: if
 * the GPU path cannot run (no device, a node without a GPU implementation) the
 * output is filled with NaN, the min/max with NaN, a message is printed to
 * stderr and fnGetLastError() returns non-zero.
 */
#ifndef FASTNOISE_GB300_C_H
#define FASTNOISE_GB300_C_H

#include <stddef.h>
#include <stdint.h>

#ifndef FASTNOISE_API
#if defined(_WIN32)
#define FASTNOISE_API __declspec(dllexport)
#else
#define FASTNOISE_API __attribute__((visibility("default")))
#endif
#endif

#ifdef __cplusplus
extern "C" {
#else
#include <stdbool.h>
#endif

/* ---------------------------------------------------------------------------
 * Part 1: reference-compatible entry points
 * ------------------------------------------------------------------------- */

/* FastNoise_C.h:27 -- decode an encoded node tree; NULL on failure.  maxFeatureSet is accepted and ignored. */
FASTNOISE_API void* fnNewFromEncodedNodeTree(const char* encodedString, unsigned maxFeatureSet);
/* FastNoise_C.h:32 -- release one reference; NULL is a no-op. */
FASTNOISE_API void fnDeleteNodeRef(void* node);
/* FastNoise_C.h:38 -- feature set of the node; this backend reports FN_GB300_FEATURE_SET. */
FASTNOISE_API unsigned fnGetActiveFeatureSet(const void* node);
/* FastNoise_C.h:44 */
FASTNOISE_API int fnGetMetadataID(const void* node);

/* FastNoise_C.h:66-80 -- out[y*xCount + x]; outputMinMax is NULL or float[2] */
FASTNOISE_API void fnGenUniformGrid2D(const void* node, float* noiseOut, float xOffset, float yOffset, int xCount,
                                      int yCount, float xStepSize, float yStepSize, int seed, float* outputMinMax);
/* FastNoise_C.h:91-106 */
FASTNOISE_API void fnGenUniformGrid3D(const void* node, float* noiseOut, float xOffset, float yOffset, float zOffset,
                                      int xCount, int yCount, int zCount, float xStepSize, float yStepSize,
                                      float zStepSize, int seed, float* outputMinMax);
/* FastNoise_C.h:120-138 */
FASTNOISE_API void fnGenUniformGrid4D(const void* node, float* noiseOut, float xOffset, float yOffset, float zOffset,
                                      float wOffset, int xCount, int yCount, int zCount, int wCount, float xStepSize,
                                      float yStepSize, float zStepSize, float wStepSize, int seed, float* outputMinMax);
/* FastNoise_C.h:164-170 */
FASTNOISE_API void fnGenPositionArray2D(const void* node, float* noiseOut, int count, const float* xPosArray,
                                        const float* yPosArray, float xOffset, float yOffset, int seed,
                                        float* outputMinMax);
/* FastNoise_C.h:193-199 */
FASTNOISE_API void fnGenPositionArray3D(const void* node, float* noiseOut, int count, const float* xPosArray,
                                        const float* yPosArray, const float* zPosArray, float xOffset, float yOffset,
                                        float zOffset, int seed, float* outputMinMax);
/* FastNoise_C.h:224-231 */
FASTNOISE_API void fnGenPositionArray4D(const void* node, float* noiseOut, int count, const float* xPosArray,
                                        const float* yPosArray, const float* zPosArray, const float* wPosArray,
                                        float xOffset, float yOffset, float zOffset, float wOffset, int seed,
                                        float* outputMinMax);
/* FastNoise_C.h:250-253 */
FASTNOISE_API void fnGenTileable2D(const void* node, float* noiseOut, int xSize, int ySize, float xStepSize,
                                   float yStepSize, int seed, float* outputMinMax);
/* FastNoise_C.h:267, 281, 298 */
FASTNOISE_API float fnGenSingle2D(const void* node, float x, float y, int seed);
FASTNOISE_API float fnGenSingle3D(const void* node, float x, float y, float z, int seed);
FASTNOISE_API float fnGenSingle4D(const void* node, float x, float y, float z, float w, int seed);

/* Metadata, FastNoise_C.h:307-651.  Invalid ids / indices return -1, false,
 * 0 or the reference's sentinel strings ("INVALID NODE ID", ...). */
FASTNOISE_API int fnGetMetadataCount(void);
FASTNOISE_API const char* fnGetMetadataName(int id);
FASTNOISE_API void* fnNewFromMetadata(int id, unsigned maxFeatureSet);
FASTNOISE_API int fnGetMetadataVariableCount(int id);
FASTNOISE_API const char* fnGetMetadataVariableName(int id, int variableIndex);
FASTNOISE_API int fnGetMetadataVariableType(int id, int variableIndex);
FASTNOISE_API int fnGetMetadataVariableDimensionIdx(int id, int variableIndex);
FASTNOISE_API int fnGetMetadataEnumCount(int id, int variableIndex);
FASTNOISE_API const char* fnGetMetadataEnumName(int id, int variableIndex, int enumIndex);
FASTNOISE_API bool fnSetVariableFloat(void* node, int variableIndex, float value);
FASTNOISE_API bool fnSetVariableIntEnum(void* node, int variableIndex, int value);
FASTNOISE_API int fnGetMetadataNodeLookupCount(int id);
FASTNOISE_API const char* fnGetMetadataNodeLookupName(int id, int nodeLookupIndex);
FASTNOISE_API int fnGetMetadataNodeLookupDimensionIdx(int id, int nodeLookupIndex);
FASTNOISE_API bool fnSetNodeLookup(void* node, int nodeLookupIndex, const void* nodeLookup);
FASTNOISE_API int fnGetMetadataHybridCount(int id);
FASTNOISE_API const char* fnGetMetadataHybridName(int id, int hybridIndex);
FASTNOISE_API int fnGetMetadataHybridDimensionIdx(int id, int hybridIndex);
FASTNOISE_API bool fnSetHybridNodeLookup(void* node, int hybridIndex, const void* nodeLookup);
FASTNOISE_API bool fnSetHybridFloat(void* node, int hybridIndex, float value);
FASTNOISE_API const char* fnGetMetadataDescription(int id);
FASTNOISE_API int fnGetMetadataGroupCount(int id);
FASTNOISE_API const char* fnGetMetadataGroupName(int id, int groupIndex);
FASTNOISE_API const char* fnGetMetadataVariableDescription(int id, int variableIndex);
FASTNOISE_API float fnGetMetadataVariableDefaultFloat(int id, int variableIndex);
FASTNOISE_API int fnGetMetadataVariableDefaultIntEnum(int id, int variableIndex);
FASTNOISE_API float fnGetMetadataVariableMinFloat(int id, int variableIndex);
FASTNOISE_API float fnGetMetadataVariableMaxFloat(int id, int variableIndex);
FASTNOISE_API const char* fnGetMetadataNodeLookupDescription(int id, int nodeLookupIndex);
FASTNOISE_API const char* fnGetMetadataHybridDescription(int id, int hybridIndex);
FASTNOISE_API float fnGetMetadataHybridDefault(int id, int hybridIndex);

/* ---------------------------------------------------------------------------
 * Part 2: additions of the GB300 backend (no reference counterpart)
 * ------------------------------------------------------------------------- */

#define FN_GB300_FEATURE_SET 0x47423330u   /* value of fnGetActiveFeatureSet */

#define FN_OK 0
#define FN_ERR_ARG (-1)           /* bad argument (null node, negative count, ...) */
#define FN_ERR_COMPILE (-2)       /* tree cannot be evaluated on the GPU (see message) */
#define FN_ERR_CUDA (-3)          /* CUDA runtime error */
#define FN_ERR_CAPACITY (-4)      /* request does not fit a pool / queue / scratch limit */
#define FN_ERR_TIMEOUT (-5)       /* a bounded wait ran out */
#define FN_ERR_STATE (-6)         /* object in the wrong state (closed server, ...) */

/* Last status of this thread (0 after a successful call), and its message. */
FASTNOISE_API int fnGetLastError(void);
FASTNOISE_API const char* fnGetLastErrorString(void);

/* Serialise like Metadata::SerialiseNodeData (reference src/FastNoise/Metadata.cpp:297-308).
 * Writes a NUL-terminated string if it fits; returns its length (excluding NUL) or a negative status. */
FASTNOISE_API int fnSerialiseNodeTree(const void* node, char* buffer, int bufferSize);

/* Read a node's members back (no counterpart in the reference, whose C++ objects hold them;
 * the C++ layer's Metadata::DeserialiseNodeData uses these).  Variables come back as the raw
 * bits of the last value set (the reference's Metadata::MemberVariable::ValueUnion); lookups
 * and hybrid nodes come back with a new reference the caller drops with fnDeleteNodeRef, or
 * NULL when unset or out of range; a hybrid's float is its constant (used while no node is set). */
FASTNOISE_API int fnGetVariableBits(const void* node, int variableIndex, int* bits);
FASTNOISE_API void* fnGetNodeLookupRef(const void* node, int nodeLookupIndex);
FASTNOISE_API void* fnGetHybridNodeLookupRef(const void* node, int hybridIndex);
FASTNOISE_API int fnGetHybridFloat(const void* node, int hybridIndex, float* value);

/* Device-pointer variants of the generation calls.  `dOut` is device memory
 * (count floats); `dMinMax` is NULL or device float[2]; `stream` is a
 * cudaStream_t (NULL = the legacy default stream, as in CUDA's own calls).
 * The call is asynchronous: it returns once the work is queued on the stream. */
FASTNOISE_API int fnGenUniformGrid2DDevice(const void* node, float* dOut, float xOffset, float yOffset, int xCount,
                                           int yCount, float xStepSize, float yStepSize, int seed, float* dMinMax,
                                           void* stream);
FASTNOISE_API int fnGenUniformGrid3DDevice(const void* node, float* dOut, float xOffset, float yOffset, float zOffset,
                                           int xCount, int yCount, int zCount, float xStepSize, float yStepSize,
                                           float zStepSize, int seed, float* dMinMax, void* stream);
FASTNOISE_API int fnGenUniformGrid4DDevice(const void* node, float* dOut, float xOffset, float yOffset, float zOffset,
                                           float wOffset, int xCount, int yCount, int zCount, int wCount,
                                           float xStepSize, float yStepSize, float zStepSize, float wStepSize, int seed,
                                           float* dMinMax, void* stream);
FASTNOISE_API int fnGenPositionArray2DDevice(const void* node, float* dOut, int count, const float* dX, const float* dY,
                                             float xOffset, float yOffset, int seed, float* dMinMax, void* stream);
FASTNOISE_API int fnGenPositionArray3DDevice(const void* node, float* dOut, int count, const float* dX, const float* dY,
                                             const float* dZ, float xOffset, float yOffset, float zOffset, int seed,
                                             float* dMinMax, void* stream);
FASTNOISE_API int fnGenPositionArray4DDevice(const void* node, float* dOut, int count, const float* dX, const float* dY,
                                             const float* dZ, const float* dW, float xOffset, float yOffset,
                                             float zOffset, float wOffset, int seed, float* dMinMax, void* stream);
FASTNOISE_API int fnGenTileable2DDevice(const void* node, float* dOut, int xSize, int ySize, float xStepSize,
                                        float yStepSize, int seed, float* dMinMax, void* stream);

/* ---- batched generation: many requests, one persistent launch ---------------------------- */

#define FN_KIND_GRID2D 0
#define FN_KIND_GRID3D 1
#define FN_KIND_GRID4D 2
#define FN_KIND_TILEABLE2D 3        /* count[0..1] = x/y size, step[0..1] = x/y step */
#define FN_KIND_POSITIONS2D 4       /* count[0] = points, positions[0..1] device arrays */
#define FN_KIND_POSITIONS3D 5
#define FN_KIND_POSITIONS4D 6

typedef struct fnGenRequest {
    const void* node;               /* tree to evaluate (any mix of trees per batch) */
    int kind;                       /* FN_KIND_* */
    int seed;
    int count[4];                   /* grid counts (x fastest) or as noted above */
    float offset[4];
    float step[4];
    const float* positions[4];      /* device arrays for FN_KIND_POSITIONS*D */
    float* out;                     /* device output, one float per point */
    float* minMax;                  /* NULL or host float[2]; filled by FN_BATCH_SYNC calls */
} fnGenRequest;

#define FN_BATCH_SYNC 1             /* wait for the batch and fill every minMax */
#define FN_BATCH_NO_GRAPH 2         /* plain stream launches instead of the captured CUDA graph */

/* Evaluate `count` requests in one persistent launch on `stream` (NULL = default stream).
 * Tile size and CTAs per SM come from the autotuner's entry for this batch's signature
 * (set by fnAutotuneBatch), else defaults. */
FASTNOISE_API int fnGenBatchDevice(const fnGenRequest* requests, int count, void* stream, int flags);
/* The same requests with HOST outputs (pinned memory gives full copy speed; any host memory
 * works): request.out points to host memory, minMax (host float[2] or NULL) is filled, and the
 * call returns when every output is on the host.  The requests are generated in slices of at
 * most 2^25 points (smaller at the start and the end) through two device staging buffers, each
 * slice's copy to the host overlapping the next slice's generation; requests whose outputs are
 * adjacent in host memory are copied together.  fnGetBatchInfo then reports the slices summed.
 * Exception: when every output lies in ordinary (pageable) memory whose pages are resident, on
 * a device that accesses pageable memory through the host's page tables (a Grace host), the
 * batch kernels store into the outputs directly (copies into pageable memory are slower);
 * FASTNOISE_HOST_DIRECT=0 turns this off.  flags: reserved, pass 0. */
FASTNOISE_API int fnGenBatchHost(const fnGenRequest* requests, int count, int flags);
/* The per-call path for the same request list: one plain launch per request, queued in
 * order on `stream` (what a caller looping over fnGen*Device would do), for comparison
 * with fnGenBatchDevice.  minMax pointers are filled when FN_BATCH_SYNC is set. */
FASTNOISE_API int fnGenEachDevice(const fnGenRequest* requests, int count, void* stream, int flags);
/* The per-call path driven by arrival times, for latency measurement beside the server:
 * requests[k] is launched as one fnGen*Device call on `stream` once arrivalMicros[k]
 * microseconds have passed since the call began (the calling thread waits in between, and
 * issues late when it falls behind), followed by a copy of its min/max to the host; a second
 * host thread waits for each request in order.  latencyMicros[k] (may be NULL) = the moment
 * the request's min/max was on the host minus its arrival time.  minMax pointers are filled.
 * Returns when every request has completed. */
FASTNOISE_API int fnGenEachPaced(const fnGenRequest* requests, int count, const double* arrivalMicros, void* stream,
                                 double* latencyMicros);
/* Tune this batch: time each tile size / CTAs-per-SM candidate on the whole batch and remember
 * the fastest for the batch's signature; then choose, for every tree of the batch that has
 * specialised kernels, a variant of its batch kernel (threads per block, register bound, points
 * in flight per thread; built here on first use, seconds): tree by tree, most points first, each
 * variant is timed on the whole batch and kept when the batch gets faster.  Later batches (and
 * the server) use both choices; fnAutotuneSave writes them out ("tree" lines for the per-tree
 * choices). */
FASTNOISE_API int fnAutotuneBatch(const fnGenRequest* requests, int count, void* stream);
FASTNOISE_API int fnAutotuneLoad(const char* path);
FASTNOISE_API int fnAutotuneSave(const char* path);

/* ---- request server: continuous batching over a device memory pool ------------------------ */

typedef struct fnServerConfig {
    unsigned long long poolBytes;   /* device pool for server-owned outputs (default 1 GiB) */
    int streams;                    /* batches in flight at once (default 3) */
    int maxBatchRequests;           /* requests per launch (default 1024) */
    long long maxBatchPoints;       /* points per launch (default 64 Mi) */
    int idleWaitMicros;             /* longest request-loop wait when no batch is in flight (default 50);
                                     * while batches are in flight the loop polls continuously */
} fnServerConfig;

typedef struct fnServerStats {
    unsigned long long submitted, completed, failed, batches, points;
    double p50Micros, p99Micros, maxMicros, meanMicros;   /* submit -> completion latency */
    unsigned long long poolUsed, poolCapacity;
    int queueDepth, inflight;
    /* Batches that were executing on the GPU at the same moment as another batch: the kernels
     * stamp each request's completion with the device clock, and two batches whose spans of
     * completions intersect were both running then. */
    unsigned long long overlappedBatches;
    int maxInflightBatches;         /* most batches launched and not yet retired at once */
    int maxConcurrentBatches;       /* most batches executing at one moment (device clock) */
} fnServerStats;

/* NULL config = defaults.  Returns NULL (error set) if the device or pool is unavailable. */
FASTNOISE_API void* fnServerCreate(const fnServerConfig* config);
/* Waits for batches in flight; requests never admitted are cancelled. */
FASTNOISE_API void fnServerDestroy(void* server);
/* Queue one request.  request->out NULL = the server allocates the output from its pool
 * (admission waits for pool memory).  Tree errors are reported here (FN_ERR_COMPILE). */
FASTNOISE_API int fnServerSubmit(void* server, const fnGenRequest* request, unsigned long long* ticket);
/* Queue `count` requests under one lock; all or nothing (nothing is queued if any request is
 * invalid).  tickets[i] receives the ticket of requests[i]. */
FASTNOISE_API int fnServerSubmitMany(void* server, const fnGenRequest* requests, int count, unsigned long long* tickets);
/* Open-loop submission: requests[k] is queued when arrivalMicros[k] microseconds have passed
 * since the call began (the calling thread waits in between); its latency in the statistics
 * counts from that arrival time.  Returns once every request is queued (all are validated
 * first; nothing is queued if any is invalid).  Use fnServerWaitMany for completion. */
FASTNOISE_API int fnServerSubmitPaced(void* server, const fnGenRequest* requests, int count,
                                      const double* arrivalMicros, unsigned long long* tickets);
/* Wait until every ticket has finished; FN_ERR_TIMEOUT when timeoutMs (>= 0) runs out first,
 * else 0 or the status of the first failed / cancelled request. */
FASTNOISE_API int fnServerWaitMany(void* server, const unsigned long long* tickets, int count, int timeoutMs);
/* 1 = done, 0 = pending, negative = failed / cancelled / unknown ticket. */
FASTNOISE_API int fnServerPoll(void* server, unsigned long long ticket);
/* Wait up to timeoutMs (negative = forever); on success fills minMax (host float[2]) and
 * *dOut (device output pointer), either may be NULL.  FN_ERR_TIMEOUT when the wait runs out. */
FASTNOISE_API int fnServerWait(void* server, unsigned long long ticket, int timeoutMs, float* minMax, float** dOut);
/* Cancel a request that has not been admitted yet (FN_ERR_STATE otherwise). */
FASTNOISE_API int fnServerCancel(void* server, unsigned long long ticket);
/* Forget a finished request and return its pool memory. */
FASTNOISE_API int fnServerRelease(void* server, unsigned long long ticket);
FASTNOISE_API int fnServerGetStats(void* server, fnServerStats* stats);
FASTNOISE_API int fnServerResetStats(void* server);

/* Compile `node` for dimensionality 2/3/4 on the host only (no CUDA call) and report the
 * program size: returns 0 and fills nInstr / nRegs (either may be NULL), or a negative status. */
FASTNOISE_API int fnCompileInfo(const void* node, int dimension, int* nInstr, int* nRegs);

/* Compile (and cache on the device) the program for `node` at dimensionality 2/3/4.
 * Generation calls do this on demand; calling it ahead moves the cost out of the first call. */
FASTNOISE_API int fnPrepare(const void* node, int dimension);

/* Shape of this thread's last fnGenBatchDevice launch (no counterpart in the reference). */
typedef struct fnBatchInfo {
    int requests;
    int specialised;                /* 1 = the fnJitCompile batch kernel ran, 0 = the interpreter */
    int tilePoints;                 /* points per work item */
    int ctas;                       /* persistent CTAs launched */
    unsigned long long workItems;   /* (request, tile) items in the device queue */
    unsigned long long points;
    unsigned long long uploadBytes; /* descriptor bytes copied host -> device for the launch */
    int kernels;                    /* kernels launched (one per tree and dimensionality when specialised) */
} fnBatchInfo;
FASTNOISE_API int fnGetBatchInfo(fnBatchInfo* info);

/* NoiseTexture::BuildTexture (no counterpart in the reference's library: its Node Editor builds
 * preview images in tools/NodeEditor/NoiseTexture.cpp:499-540).  The tree is wrapped in a
 * default ConvertRGBA8 (range -1..1 to grey 0..255, alpha 255) and generated over sizeX x sizeY
 * pixels centred on (offset[0], offset[1]), `scale` apart: genType 0 = 2D grid, 1 = 2D
 * tileable, 2 = 3D slice at z = offset[2], 3 = 4D slice at (offset[2], offset[3]).  dPixels:
 * device uint32[sizeX * sizeY], row-major, written by the generation kernel itself (4 bytes per
 * pixel, no float image in between); dMinMax (device float[2] or NULL) receives the
 * OutputMinMax of the packed values, as the editor's call returns it.  Asynchronous. */
FASTNOISE_API int fnGenPreviewTextureDevice(const void* node, int genType, int sizeX, int sizeY, const float* offset,
                                            float scale, int seed, unsigned int* dPixels, float* dMinMax, void* stream);

/* Chunk meshing after the noise (no counterpart in the reference's library: its Node Editor
 * meshes preview chunks on the CPU in tools/NodeEditor/MeshNoisePreview.cpp, with a chunk size
 * of 128).  The chunk's densities are generated on the GPU exactly as the editor's
 * GenPositionArray3D/2D calls do, then meshed on the GPU; vertices and indices come out in the
 * editor's order.  vertices / indices are device buffers; the call is synchronous and fills
 * the counts, heights and OutputMinMax, returning FN_ERR_CAPACITY (counts filled) when the
 * buffers are too small. */
typedef struct fnMeshVertex { float x, y, z, light; } fnMeshVertex;   /* the editor's VertexData */
typedef struct fnChunkMesh {
    fnMeshVertex* vertices;         /* device, vertexCapacity entries */
    unsigned int* indices;          /* device, indexCapacity entries (triangle list) */
    int vertexCapacity, indexCapacity;
    int vertexCount, indexCount;    /* out: the whole mesh (also when it did not fit) */
    float minAirY, maxSolidY;       /* out (bloxel, dmc): lowest air / highest solid height, +-inf if none */
    float minMax[2];                /* out: OutputMinMax of the densities */
} fnChunkMesh;
/* Where the chunk meshers keep a chunk's densities (no counterpart in the reference).
 * FN_MESH_DENSITY_ARRAY (default): the tree's kernel writes every density of the chunk into a
 * device array that the mesher passes read ((size+2)^3 or (size+4)^3 floats; for the editor's
 * 128^3 chunks 9 MB, which stays in L2).  FN_MESH_DENSITY_SPARSE: for trees with specialised
 * kernels the densities never leave registers; the tree's kernel stores only their
 * classification against the iso level (2 bits each), and the exact values the light and
 * vertex passes read are evaluated again at those voxels only (the bloxel mesher's surface
 * voxels; a gradient stencil around every dual marching cubes vertex).  Same meshes bit for
 * bit; the array form measures faster on a GB300.  Returns the previous setting (or
 * FN_ERR_ARG). */
#define FN_MESH_DENSITY_ARRAY 0
#define FN_MESH_DENSITY_SPARSE 1
FASTNOISE_API int fnSetMeshDensityForm(int form);
/* BuildBloxel3DMesh (MeshNoisePreview.cpp:443-590): block faces between solid (density <=
 * isoSurface) and air voxels of a size^3 chunk at (posX, posY, posZ), with ambient occlusion
 * and directional light; size <= 256 (every index fits 32 bits).  upAxisZ swaps the y and z noise axes. */
FASTNOISE_API int fnBuildChunkMeshBloxel(const void* node, int size, int posX, int posY, int posZ, int seed,
                                         float isoSurface, int upAxisZ, fnChunkMesh* mesh, void* stream);
/* BuildDmc3DMesh / DmcGetVertIndex (MeshNoisePreview.cpp:592-953), the editor's default mesh:
 * dual marching cubes over a size^3 chunk at (posX, posY, posZ) with a two-voxel apron, one
 * vertex per surface piece of each cell (the mean of its edge crossings, lit by the density
 * gradient), one quad per cut grid edge, vertices shared and numbered in the editor's first-use
 * order; size <= 256.  Vertices and indices are written only when both fit. */
FASTNOISE_API int fnBuildChunkMeshDmc(const void* node, int size, int posX, int posY, int posZ, int seed,
                                      float isoSurface, int upAxisZ, fnChunkMesh* mesh, void* stream);
/* Many chunks of one tree in one call (what the editor's mesh worker threads do chunk by
 * chunk): positions holds (x, y, z) per chunk, meshes one fnChunkMesh per chunk, each with its
 * own buffers.  The chunks run on several internal streams, ordered after earlier work on
 * `stream`; the call returns when every chunk is done.  FN_ERR_CAPACITY when any chunk's
 * buffers were too small (that chunk's counts are filled; the others are complete). */
FASTNOISE_API int fnBuildChunkMeshesBloxel(const void* node, int size, int count, const int* positions, int seed,
                                           float isoSurface, int upAxisZ, fnChunkMesh* meshes, void* stream);
FASTNOISE_API int fnBuildChunkMeshesDmc(const void* node, int size, int count, const int* positions, int seed,
                                        float isoSurface, int upAxisZ, fnChunkMesh* meshes, void* stream);
/* BuildHeightMap2DMesh (MeshNoisePreview.cpp:956-1004): size^2 quads of a 2D heightmap at
 * (posX, posZ), heights = density * heightMultiplier; size <= 8192. */
FASTNOISE_API int fnBuildChunkMeshHeightmap(const void* node, int size, int posX, int posZ, int seed,
                                            float heightMultiplier, fnChunkMesh* mesh, void* stream);

/* Live trees (no counterpart in the reference, whose consumers poll the Node Editor's channel,
 * tools/NodeEditorIpc, and rebuild their generator themselves).  A live tree follows a channel
 * from fnEditorIpcSetup (NodeEditorIpc_C.h): fnLiveTreeUpdate polls it and, for each tree the
 * editor sends as its selected node, decodes it, compiles it for the listed dimensionalities
 * (and specialises it with NVRTC when specialisation is enabled), and only then makes it
 * current, so callers never wait on or see a half-built tree.  A tree that fails to decode or
 * compile is rejected and the current one stays.  With pollMs > 0 a background thread updates
 * every pollMs milliseconds (the live tree then owns polling of that channel).  ipc may be NULL
 * (the initial tree only).  fnLiveTreeUpdate returns 1 when a new tree became current, 0 when
 * nothing new arrived, FN_ERR_* when the newest tree was rejected.  fnLiveTreeAcquire returns
 * the current tree with a reference the caller drops with fnDeleteNodeRef (NULL before the
 * first tree); requests already submitted keep the tree they were submitted with. */
typedef struct fnLiveTreeInfo {
    unsigned long long version;     /* trees made current so far */
    unsigned long long rejected;    /* trees that failed to decode or compile */
    int lastStatus;                 /* FN_OK, or the FN_ERR_* of the last rejected tree */
    char lastError[256];
} fnLiveTreeInfo;
FASTNOISE_API void* fnLiveTreeCreate(void* ipc, const char* initialEncodedTree, const int* dimensions, int count, int pollMs);
FASTNOISE_API int fnLiveTreeUpdate(void* live);
FASTNOISE_API void* fnLiveTreeAcquire(void* live, unsigned long long* version);
FASTNOISE_API int fnLiveTreeGetInfo(void* live, fnLiveTreeInfo* info);
FASTNOISE_API void fnLiveTreeDelete(void* live);

/* Run-time specialisation (no counterpart in the reference, whose trees run through
 * virtual calls per SIMD block).  Each (node, dimension) pair is compiled to straight-line
 * CUDA and built for sm_103a with NVRTC: per-tree kernels for the grid, position-array and
 * tileable calls, and a persistent batch kernel per tree.  Later generation calls on these
 * trees (host, device, batch and server paths) use the specialised kernels; results are
 * bit-identical to the interpreter's.  Building takes seconds, so do it once at start-up.
 * Kernels of earlier calls stay loaded (a tree specialised again gets its new kernels).
 * Returns FN_OK or FN_ERR_*. */
FASTNOISE_API int fnJitCompile(const void* const* nodes, const int* dimensions, int count);
/* Automatic specialisation: a tree that has run `uses` times on the program interpreter (per
 * dimensionality; host, device, batch and server calls all count) is specialised on a
 * background thread, and its later calls use the specialised kernels -- the same results,
 * without a call to fnJitCompile.  0 turns it off; the default is 4, or the number in the
 * environment variable FASTNOISE_AUTO_SPECIALISE.  Returns the previous setting. */
FASTNOISE_API int fnSetAutoSpecialise(int uses);
/* Wait until no background specialisation is queued or running (timeoutMs < 0: no limit);
 * FN_OK, or FN_ERR_TIMEOUT. */
FASTNOISE_API int fnAutoSpecialiseWait(int timeoutMs);
/* 1 when the tree's specialised kernels for `dimension` are loaded, 0 when calls run on the
 * interpreter, FN_ERR_* on error. */
FASTNOISE_API int fnJitIsSpecialised(const void* node, int dimension);
/* On-disk cache of the specialised modules: each compiled module is kept in a directory,
 * keyed by its CUDA source, the NVRTC options and the NVRTC version.  A later process loads
 * it instead of compiling (milliseconds instead of seconds), and a tree that an earlier
 * process specialised alone (as automatic specialisation does) runs its specialised kernels
 * from its first call, without interpreted calls.  Off by default (the library writes no
 * files of its own); the environment variable FASTNOISE_JIT_CACHE names a directory, created
 * if missing, and fnJitSetCacheDir sets or replaces it for this process (NULL, "" or "off":
 * off).
 * fnJitGetCacheInfo copies the directory in use into dir (dirBytes with the terminating zero;
 * dir may be NULL), fills this process's cache hits and misses (either may be NULL), and
 * returns the directory's length (0 = off). */
FASTNOISE_API int fnJitSetCacheDir(const char* dir);
FASTNOISE_API int fnJitGetCacheInfo(char* dir, int dirBytes, unsigned long long* hits, unsigned long long* misses);
/* Generate and compile the module source with NVRTC without loading it (no GPU needed);
 * *cubinBytes (may be NULL) receives the size of the compiled code. */
FASTNOISE_API int fnJitCheck(const void* const* nodes, const int* dimensions, int count, int* cubinBytes);
/* The same for the other variants of the trees' batch kernels (block size, register bound,
 * points in flight per thread), which fnAutotuneBatch builds and times per tree. */
FASTNOISE_API int fnJitCheckBatchVariants(const void* const* nodes, const int* dimensions, int count, int* cubinBytes);
/* Turn the use of specialised kernels on (1, the default) or off (0, interpreter only).
 * Returns the previous setting. */
FASTNOISE_API int fnSetJitEnabled(int enabled);

/* No counterpart in the reference.  fnGenUniformGrid3DDevice for callers that
 * cannot let the library allocate device memory: applications whose own pool
 * allocator takes all device memory at start-up (a library cudaMalloc would then
 * fail or shrink the pool), and frame loops with a fixed time budget that cannot
 * absorb the device-wide synchronisation of cudaFree.  It calls no cudaMalloc /
 * cudaFree / cudaMallocHost and creates no stream: the tree's program and the
 * min/max workspace live in one fixed-size static device array per device,
 * filled by stream-ordered copies on `stream`.
 * - NULL stream: the legacy default stream, as for fnGenUniformGrid3DDevice.
 * - Limit: the tree's compiled program must fit 16 KiB (several hundred nodes);
 *   larger trees return FN_ERR_CAPACITY without touching the GPU.
 * - Not for use while `stream` is being captured into a CUDA graph: each call
 *   uploads the program from pageable host memory that the next call reuses.
 * - Every call shares the array and it keeps the last call's contents; calls
 *   ordered on one stream are safe, calls that overlap on the GPU (different
 *   streams without ordering between them) race and give wrong results.
 * The other arguments, the outputs and the asynchronous behaviour are those of
 * fnGenUniformGrid3DDevice. */
FASTNOISE_API int fnGenUniformGrid3DDeviceNoAlloc(const void* node, float* dOut, float xOffset, float yOffset,
                                                  float zOffset, int xCount, int yCount, int zCount, float xStepSize,
                                                  float yStepSize, float zStepSize, int seed, float* dMinMax,
                                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FASTNOISE_GB300_C_H */
