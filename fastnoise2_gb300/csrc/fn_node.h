// fn_node.h -- host-side FastNoise2 node model.
//
// Mirrors the reference's object model at the level the drop-in boundary needs:
//  * node registry with the reference ids (registration order,
//    src/FastNoise/FastSIMD_Build.inl:86-143) and member lists in metadata order
//    (include/FastNoise/Generators/<Node>.h MetadataT<> constructors);
//  * member setters with the reference's side effects (ScalableGenerator::SetScale,
//    VariableRange::SetOutputMin/Max, Terrace::SetSmoothness, DomainRotate ...);
//  * intrusive reference counting (Generator.inl:512-522, SmartNode.h:71-320);
//  * encoded node trees: Metadata::SerialiseNodeData / NewFromEncodedNodeTree
//    (src/FastNoise/Metadata.cpp:88-506) and Base64 with '@' runs (Base64.h).
#pragma once
#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

namespace fn {

enum NodeId : int {
    kConstant = 0, kWhite, kCheckerboard, kSineWave, kGradient, kDistanceToPoint,
    kSimplex, kSuperSimplex, kPerlin, kValue,
    kCellularValue, kCellularDistance, kCellularLookup,
    kFractalFBm, kPingPong, kFractalRidged,
    kDomainWarpSimplex, kDomainWarpSuperSimplex, kDomainWarpGradient,
    kDomainWarpFractalProgressive, kDomainWarpFractalIndependent,
    kAdd, kSubtract, kMultiply, kDivide,
    kAbs, kMin, kMax, kMinSmooth, kMaxSmooth, kSignedSquareRoot, kPowFloat, kPowInt,
    kDomainScale, kDomainOffset, kDomainRotate, kDomainAxisScale,
    kSeedOffset, kConvertRGBA8, kGeneratorCache,
    kFade, kRemap, kTerrace, kAddDimension, kRemoveDimension,
    kModulus, kDomainRotatePlane,
    kNodeCount
};

enum VarType : int { kVarFloat = 0, kVarInt = 1, kVarEnum = 2 };   // Metadata.h:68-73

// What a member-variable setter does to the node state.
enum SetterKind : int {
    S_NONE = 0, S_SCALE, S_SEED, S_OUT_MIN, S_OUT_MAX, S_VALUE, S_MULT,
    S_DIST_FUNC, S_VALUE_INDEX, S_DIST_IDX0, S_DIST_IDX1, S_RETURN_TYPE,
    S_OCTAVES, S_LACUNARITY, S_AXIS, S_VEC_SCHEME, S_POW_INT, S_DOMAIN_SCALE,
    S_YAW, S_PITCH, S_ROLL, S_SEED_OFFSET_NODE, S_RGBA_MIN, S_RGBA_MAX,
    S_INTERP, S_CLAMP, S_STEPS, S_REMOVE_DIM, S_ROT_TYPE
};

struct VarMeta {
    const char* name;
    VarType type;
    int32_t def;        // raw ValueUnion bits
    int32_t vmin;
    int32_t vmax;
    std::vector<const char*> enums;
    int dim;            // -1 unless per-dimension
    SetterKind setter;
    const char* description;
};

struct LookupMeta {
    const char* name;
    int dim;
    bool warp_only;     // GeneratorSourceT<DomainWarp>
    const char* description;
};

struct HybridMeta {
    const char* name;
    float def;
    int dim;
    const char* description;
};

struct NodeMeta {
    int id;
    const char* name;
    const char* description;
    std::vector<const char*> groups;
    std::vector<VarMeta> vars;
    std::vector<LookupMeta> lookups;
    std::vector<HybridMeta> hybrids;
};

const std::vector<NodeMeta>& all_meta();
const NodeMeta* meta_by_id(int id);
const NodeMeta* meta_by_name(const char* name);
bool is_domain_warp(int id);

// Member state exactly as the reference's setters leave it.
struct NodeState {
    float scale = 100.0f, frequency = 1.0f / 100;       // BasicGenerators.h:27-28
    int seed_offset = 0;
    float range_min = -1.0f, range_scale = 2.0f;        // BasicGenerators.h:111-112
    float value = 1.0f;
    float multiplier[4] = {0, 0, 0, 0};
    float axis[4] = {1, 1, 1, 1};
    int dist_func = 1;                                  // EuclideanSquared (Cellular.h:26, BasicGenerators.h:289)
    int value_index = 0, dist_idx0 = 0, dist_idx1 = 1, return_type = 0;
    int octaves = 3;
    float lacunarity = 2.0f;
    int vec_scheme = 0;
    int pow_int = 2;
    float dscale = 1.0f;
    float yaw_cos = 1, yaw_sin = 0, pitch_cos = 1, pitch_sin = 0, roll_cos = 1, roll_sin = 0;
    float rot[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    float rgba_min = -1.0f, rgba_max = 1.0f;
    int interp = 0, clamp_output = 0;
    float step_count = 1.0f, step_recip = 1.0f, smooth_recip = 0.0f;
    int remove_dim = 1;
    int rot_type = 0;
};

class Node {
public:
    explicit Node(const NodeMeta* meta);
    ~Node();
    Node(const Node&) = delete;
    Node& operator=(const Node&) = delete;

    const NodeMeta* meta;
    std::atomic<int32_t> refs{0};
    std::vector<int32_t> vars;            // NodeData view: raw bits as last set
    std::vector<Node*> lookups;           // counted references
    std::vector<Node*> hnodes;            // counted references (nullptr = constant)
    std::vector<float> hvals;
    NodeState st;

    // Reference setter semantics.  Return false where the reference's
    // metadata setFunc returns false (index out of range, wrong node type).
    bool set_var(int idx, int32_t bits);
    bool set_lookup(int idx, Node* child);
    bool set_hybrid_node(int idx, Node* child);
    bool set_hybrid_float(int idx, float v);
    bool lookup_accepts(int idx, const Node* child) const;
};

void node_ref(Node* n);
void node_unref(Node* n);
Node* node_new(int id);                   // refs = 1

// Bumped by every setter; used to skip recompiling unchanged trees.
uint64_t mutation_epoch();

// Base64 with '@' run-length compression of 'A' (Base64.h)
std::string base64_encode(const std::vector<uint8_t>& data);
std::vector<uint8_t> base64_decode(const char* text);

// Returns a node with refs = 1, or nullptr where the reference returns nullptr.
Node* decode_tree(const char* encoded);
// Serialise like Metadata::SerialiseNodeData (non-default variables only,
// back-references for shared nodes).  Empty string on failure.
std::string encode_tree(const Node* root);

}  // namespace fn
