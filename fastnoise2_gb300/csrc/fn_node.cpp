// fn_node.cpp -- node registry, setters, reference counting and the encoded
// node-tree codec.  See fn_node.h for the reference files each part follows.
#include "fn_node.h"

#include <cmath>
#include <cstring>
#include <unordered_map>

namespace fn {

namespace {

int32_t fbits(float f) { int32_t i; std::memcpy(&i, &f, 4); return i; }
float bitsf(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }

std::atomic<uint64_t> g_epoch{1};

const std::vector<const char*> kDistFunc = {"Euclidean", "Euclidean Squared", "Manhattan", "Hybrid", "Max Axis", "Minkowski"};
const std::vector<const char*> kBoolean = {"False", "True"};
const std::vector<const char*> kDims = {"X", "Y", "Z", "W"};
const std::vector<const char*> kReturnType = {"Index0", "Index0Add1", "Index0Sub1", "Index0Mul1", "Index0Div1"};
const std::vector<const char*> kInterp = {"Linear", "Hermite", "Quintic"};
const std::vector<const char*> kVecScheme = {"Orthogonal Gradient Matrix", "Gradient Outer Product"};
const std::vector<const char*> kPlaneRot = {"Improve XY Planes", "Improve XZ Planes"};

VarMeta vf(const char* name, float def, SetterKind s, const char* desc = "", int dim = -1)
{
    return VarMeta{name, kVarFloat, fbits(def), fbits(0.0f), fbits(0.0f), {}, dim, s, desc};
}
VarMeta vi(const char* name, int def, SetterKind s, int lo = 0, int hi = 0, const char* desc = "")
{
    return VarMeta{name, kVarInt, def, lo, hi, {}, -1, s, desc};
}
VarMeta ve(const char* name, int def, const std::vector<const char*>& names, SetterKind s, const char* desc = "")
{
    return VarMeta{name, kVarEnum, def, 0, 0, names, -1, s, desc};
}

std::vector<VarMeta> cat(std::initializer_list<std::vector<VarMeta>> parts)
{
    std::vector<VarMeta> out;
    for (auto& p : parts) out.insert(out.end(), p.begin(), p.end());
    return out;
}
std::vector<VarMeta> per_dim_var(const char* name, float def, SetterKind s, const char* desc)
{
    std::vector<VarMeta> out;
    for (int k = 0; k < 4; ++k) out.push_back(vf(name, def, s, desc, k));
    return out;
}
std::vector<HybridMeta> per_dim_hyb(const char* name, float def, const char* desc)
{
    std::vector<HybridMeta> out;
    for (int k = 0; k < 4; ++k) out.push_back(HybridMeta{name, def, k, desc});
    return out;
}
template <class T>
std::vector<T> cat2(std::vector<T> a, const std::vector<T>& b)
{
    a.insert(a.end(), b.begin(), b.end());
    return a;
}

std::vector<NodeMeta> build_meta()
{
    // Member chains: ScalableGenerator, Seeded<>, VariableRange<> (BasicGenerators.h:37,73,121-122)
    const std::vector<VarMeta> scale = {vf("Feature Scale", 100.0f, S_SCALE, "Size of one noise feature in world units (1 / frequency)")};
    const std::vector<VarMeta> seed = {vi("Seed Offset", 0, S_SEED, 0, 0, "Added to this node's seed only; child nodes keep the incoming seed")};
    const std::vector<VarMeta> range = {vf("Output Min", -1.0f, S_OUT_MIN, "Lower end of the output range"),
                                        vf("Output Max", 1.0f, S_OUT_MAX, "Upper end of the output range")};
    const std::vector<VarMeta> noise = cat({scale, seed, range});
    const VarMeta cellDf = ve("Distance Function", 1, kDistFunc, S_DIST_FUNC, "Metric used to find the nearest cells");
    const std::vector<HybridMeta> cellH = {
        {"Minkowski P", 1.5f, -1, "Exponent of the Minkowski metric (1 = Manhattan, 2 = Euclidean)"},
        {"Grid Jitter", 1.0f, -1, "How far cell points move away from the regular grid"},
        {"Size Jitter", 0.0f, -1, "Random per-cell distance multiplier"}};
    const std::vector<HybridMeta> fractH = {
        {"Gain", 0.5f, -1, "Amplitude multiplier from one octave to the next"},
        {"Weighted Strength", 0.0f, -1, "Lets the previous octave's value scale the next octave's amplitude"}};
    const std::vector<VarMeta> fractV = {vi("Octaves", 3, S_OCTAVES, 2, 16, "Number of layers combined"),
                                         vf("Lacunarity", 2.0f, S_LACUNARITY, "Frequency multiplier between octaves")};
    const std::vector<VarMeta> warpV = cat({scale, seed, per_dim_var("Amplitude Scaling", 1.0f, S_AXIS, "Per-axis multiplier of the warp amplitude")});
    const std::vector<HybridMeta> warpH = {{"Warp Amplitude", 50.0f, -1, "Largest distance a position is moved"}};
    const LookupMeta src = {"Source", -1, false, "Input node"};
    const LookupMeta lhs = {"LHS", -1, false, "Left operand"};
    const HybridMeta rhs = {"RHS", 0.0f, -1, "Right operand"};
    const HybridMeta lhsH = {"LHS", 0.0f, -1, "Left operand"};

    std::vector<NodeMeta> m;
    auto add = [&](const char* name, const char* desc, std::vector<const char*> groups, std::vector<VarMeta> vars,
                   std::vector<LookupMeta> lookups, std::vector<HybridMeta> hybrids) {
        m.push_back(NodeMeta{(int)m.size(), name, desc, groups, vars, lookups, hybrids});
    };
    add("Constant", "Returns the same value everywhere", {"Basic Generators"}, {vf("Value", 1.0f, S_VALUE, "Output value")}, {}, {});
    add("White", "Uncorrelated hash noise of the input position's bits", {"Basic Generators"}, cat({seed, range}), {}, {});
    add("Checkerboard", "Alternating -1/1 cells, one cell per Feature Scale", {"Basic Generators"}, cat({scale, range}), {}, {});
    add("SineWave", "Product of per-axis sine waves", {"Basic Generators"}, cat({scale, range}), {}, {});
    add("Gradient", "Sum over axes of (position + offset) * multiplier", {"Basic Generators"},
        per_dim_var("Multiplier", 0.0f, S_MULT, "Per-axis slope"), {}, per_dim_hyb("Offset", 0.0f, "Per-axis offset"));
    add("DistanceToPoint", "Distance from the position to a fixed point", {"Basic Generators"},
        {ve("Distance Function", 0, kDistFunc, S_DIST_FUNC, "Distance metric")}, {},
        cat2(per_dim_hyb("Point", 0.0f, "Point coordinate"), {{"Minkowski P", 1.5f, -1, "Exponent of the Minkowski metric"}}));
    add("Simplex", "Simplex gradient noise", {"Coherent Noise"}, noise, {}, {});
    add("SuperSimplex", "OpenSimplex2S gradient noise", {"Coherent Noise"}, noise, {}, {});
    add("Perlin", "Classic Perlin gradient noise", {"Coherent Noise"}, noise, {}, {});
    add("Value", "Interpolated lattice value noise", {"Coherent Noise"}, noise, {}, {});
    add("CellularValue", "Hash value of the Nth closest cell", {"Coherent Noise"},
        cat({noise, {cellDf, vi("Value Index", 0, S_VALUE_INDEX, 0, 3, "Which closest cell (0 = nearest)")}}), {}, cellH);
    add("CellularDistance", "Distances to the closest cells, combined", {"Coherent Noise"},
        cat({noise, {cellDf, vi("Distance Index 0", 0, S_DIST_IDX0, 0, 3, "First distance rank"),
                     vi("Distance Index 1", 1, S_DIST_IDX1, 0, 3, "Second distance rank"),
                     ve("Return Type", 0, kReturnType, S_RETURN_TYPE, "How the two distances combine")}}), {}, cellH);
    add("CellularLookup", "Evaluates the lookup node at the closest cell point", {"Coherent Noise"}, cat({scale, seed, {cellDf}}),
        {{"Lookup", -1, false, "Node sampled at the cell point"}}, cellH);
    add("FractalFBm", "Fractional Brownian motion over the source", {"Fractal"}, fractV, {src}, fractH);
    add("PingPong", "Folds the scaled source back and forth in [0, 1]", {"Modifiers"}, {}, {src},
        {{"Ping Pong Strength", 2.0f, -1, "Scale applied before folding"}});
    add("FractalRidged", "Ridged multifractal over the source", {"Fractal"}, fractV, {src}, fractH);
    add("DomainWarpSimplex", "Simplex-based vector warp of the input position", {"Domain Warp"},
        cat({warpV, {ve("Vectorization Scheme", 0, kVecScheme, S_VEC_SCHEME, "How the scalar noise becomes a vector")}}), {src}, warpH);
    add("DomainWarpSuperSimplex", "OpenSimplex2S-based vector warp of the input position", {"Domain Warp"},
        cat({warpV, {ve("Vectorization Scheme", 0, kVecScheme, S_VEC_SCHEME, "How the scalar noise becomes a vector")}}), {src}, warpH);
    add("DomainWarpGradient", "Lattice-gradient warp of the input position", {"Domain Warp"}, warpV, {src}, warpH);
    const LookupMeta dws = {"Domain Warp Source", -1, true, "Domain warp node applied per octave"};
    add("DomainWarpFractalProgressive", "Each octave warps the previous octave's output position", {"Domain Warp", "Fractal"},
        fractV, {dws}, fractH);
    add("DomainWarpFractalIndependent", "Every octave warps the original position; offsets accumulate", {"Domain Warp", "Fractal"},
        fractV, {dws}, fractH);
    add("Add", "LHS + RHS", {"Operators"}, {}, {lhs}, {rhs});
    add("Subtract", "LHS - RHS", {"Operators"}, {}, {}, {lhsH, rhs});
    add("Multiply", "LHS * RHS", {"Operators"}, {}, {lhs}, {rhs});
    add("Divide", "LHS / RHS", {"Operators"}, {}, {}, {lhsH, rhs});
    add("Abs", "Absolute value of the source", {"Modifiers"}, {}, {src}, {});
    add("Min", "Smaller of LHS and RHS", {"Blends"}, {}, {lhs}, {rhs});
    add("Max", "Larger of LHS and RHS", {"Blends"}, {}, {lhs}, {rhs});
    add("MinSmooth", "Smooth minimum of LHS and RHS", {"Blends"}, {}, {lhs}, {rhs, {"Smoothness", 0.1f, -1, "Blend radius"}});
    add("MaxSmooth", "Smooth maximum of LHS and RHS", {"Blends"}, {}, {lhs}, {rhs, {"Smoothness", 0.1f, -1, "Blend radius"}});
    add("SignedSquareRoot", "sqrt(|x|) with the sign of x", {"Modifiers"}, {}, {src}, {});
    add("PowFloat", "Value raised to a real power", {"Blends"}, {}, {}, {{"Value", 2.0f, -1, "Base"}, {"Pow", 2.0f, -1, "Exponent"}});
    add("PowInt", "Value raised to an integer power", {"Blends"}, {vi("Pow", 2, S_POW_INT, 2, 0, "Exponent")},
        {{"Value", -1, false, "Base"}}, {});
    add("DomainScale", "Scales the input position", {"Domain Modifiers"}, {vf("Scaling", 1.0f, S_DOMAIN_SCALE, "Position multiplier")}, {src}, {});
    add("DomainOffset", "Offsets the input position", {"Domain Modifiers"}, {}, {src}, per_dim_hyb("Offset", 0.0f, "Per-axis offset"));
    add("DomainRotate", "Rotates the input position (yaw, pitch, roll in radians)", {"Domain Modifiers"},
        {vf("Yaw", 0.0f, S_YAW, "Rotation about Z"), vf("Pitch", 0.0f, S_PITCH, "Rotation about Y"), vf("Roll", 0.0f, S_ROLL, "Rotation about X")},
        {src}, {});
    add("DomainAxisScale", "Scales each axis of the input position", {"Domain Modifiers"},
        per_dim_var("Scaling", 1.0f, S_AXIS, "Per-axis multiplier"), {src}, {});
    add("SeedOffset", "Offsets the seed passed to the source", {"Modifiers"}, {vi("Seed Offset", 1, S_SEED_OFFSET_NODE, 0, 0, "Seed delta")}, {src}, {});
    add("ConvertRGBA8", "Packs the clamped source into a grey RGBA8 value", {"Modifiers"},
        {vf("Min", -1.0f, S_RGBA_MIN, "Value mapped to 0"), vf("Max", 1.0f, S_RGBA_MAX, "Value mapped to 255")}, {src}, {});
    add("GeneratorCache", "Passes the source through (results are recomputed per use)", {"Modifiers"}, {}, {src}, {});
    add("Fade", "Linear blend from A to B", {"Blends"}, {ve("Interpolation", 0, kInterp, S_INTERP, "Easing applied to the fade")},
        {{"A", -1, false, "From"}, {"B", -1, false, "To"}},
        {{"Fade", 0.0f, -1, "Blend position"}, {"Fade Min", -1.0f, -1, "Fade value giving A"}, {"Fade Max", 1.0f, -1, "Fade value giving B"}});
    add("Remap", "Maps the source range onto a new range", {"Modifiers"}, {ve("Clamp Output", 0, kBoolean, S_CLAMP, "Clamp to the new range")},
        {src}, {{"From Min", -1.0f, -1, ""}, {"From Max", 1.0f, -1, ""}, {"To Min", 0.0f, -1, ""}, {"To Max", 1.0f, -1, ""}});
    add("Terrace", "Quantises the source into steps", {"Modifiers"}, {vf("Step Count", 1.0f, S_STEPS, "Steps per unit")}, {src},
        {{"Smoothness", 0.0f, -1, "Softens the step edges"}});
    add("AddDimension", "Appends a coordinate to the input position", {"Domain Modifiers"}, {}, {src},
        {{"New Dimension Position", 0.0f, -1, "Value of the new coordinate"}});
    add("RemoveDimension", "Drops one coordinate of the input position", {"Domain Modifiers"},
        {ve("Remove Dimension", 1, kDims, S_REMOVE_DIM, "Axis removed")}, {src}, {});
    add("Modulus", "LHS modulo RHS", {"Operators"}, {}, {}, {lhsH, rhs});
    add("DomainRotatePlane", "Rotation that removes the lattice's axis alignment in one plane", {"Domain Modifiers"},
        {ve("Rotation Type", 0, kPlaneRot, S_ROT_TYPE, "Plane kept axis-free")}, {src}, {});
    return m;
}

}  // namespace

const std::vector<NodeMeta>& all_meta()
{
    static const std::vector<NodeMeta> table = build_meta();
    return table;
}

const NodeMeta* meta_by_id(int id)
{
    const auto& t = all_meta();
    return (id >= 0 && id < (int)t.size()) ? &t[id] : nullptr;
}

const NodeMeta* meta_by_name(const char* name)
{
    for (const auto& m : all_meta())
        if (std::strcmp(m.name, name) == 0) return &m;
    return nullptr;
}

bool is_domain_warp(int id)
{
    return id == kDomainWarpSimplex || id == kDomainWarpSuperSimplex || id == kDomainWarpGradient;
}

uint64_t mutation_epoch() { return g_epoch.load(std::memory_order_acquire); }

// ------------------------------------------------------------------ Node

Node::Node(const NodeMeta* m) : meta(m)
{
    for (const auto& v : m->vars) vars.push_back(v.def);
    lookups.assign(m->lookups.size(), nullptr);
    hnodes.assign(m->hybrids.size(), nullptr);
    for (const auto& h : m->hybrids) hvals.push_back(h.def);
    if (m->id == kSeedOffset) st.seed_offset = 1;               // Modifiers.h:149
    g_epoch.fetch_add(1, std::memory_order_acq_rel);            // a new node may reuse a freed address
}

Node::~Node()
{
    g_epoch.fetch_add(1, std::memory_order_acq_rel);
    for (Node* c : lookups) if (c) node_unref(c);
    for (Node* c : hnodes) if (c) node_unref(c);
}

void node_ref(Node* n) { if (n) n->refs.fetch_add(1, std::memory_order_relaxed); }

void node_unref(Node* n)
{
    if (n && n->refs.fetch_sub(1, std::memory_order_acq_rel) == 1) delete n;
}

Node* node_new(int id)
{
    const NodeMeta* m = meta_by_id(id);
    if (!m) return nullptr;
    Node* n = new Node(m);
    n->refs.store(1);
    return n;
}

static void calc_rotation(NodeState& s)   // DomainRotate::CalculateRotation (Modifiers.h:104-117)
{
    s.rot[0] = s.yaw_cos * s.pitch_cos;
    s.rot[1] = s.yaw_cos * s.pitch_sin * s.roll_sin - s.yaw_sin * s.roll_cos;
    s.rot[2] = s.yaw_cos * s.pitch_sin * s.roll_cos + s.yaw_sin * s.roll_sin;
    s.rot[3] = s.yaw_sin * s.pitch_cos;
    s.rot[4] = s.yaw_sin * s.pitch_sin * s.roll_sin + s.yaw_cos * s.roll_cos;
    s.rot[5] = s.yaw_sin * s.pitch_sin * s.roll_cos - s.yaw_cos * s.roll_sin;
    s.rot[6] = -s.pitch_sin;
    s.rot[7] = s.pitch_cos * s.roll_sin;
    s.rot[8] = s.pitch_cos * s.roll_cos;
}

static int clamp_idx(int v) { return v < 0 ? 0 : (v > 3 ? 3 : v); }

bool Node::set_var(int idx, int32_t bits)
{
    if (idx < 0 || idx >= (int)meta->vars.size()) return false;
    const VarMeta& vm = meta->vars[idx];
    vars[idx] = bits;
    const float f = bitsf(bits);
    const int i = bits;
    NodeState& s = st;
    switch (vm.setter) {
    case S_SCALE: s.scale = f; s.frequency = 1.0f / f; break;                 // BasicGenerators.h:20-24
    case S_SEED: s.seed_offset = i; break;
    case S_OUT_MIN: s.range_scale += s.range_min - f; s.range_min = f; break; // BasicGenerators.h:96-100
    case S_OUT_MAX: s.range_scale = (f - s.range_min); break;                 // BasicGenerators.h:105-108
    case S_VALUE: s.value = f; break;
    case S_MULT: s.multiplier[vm.dim] = f; break;
    case S_DIST_FUNC: s.dist_func = i; break;
    case S_VALUE_INDEX: s.value_index = clamp_idx(i); break;                  // Cellular.h:65
    case S_DIST_IDX0: s.dist_idx0 = clamp_idx(i); break;                      // Cellular.h:104-105
    case S_DIST_IDX1: s.dist_idx1 = clamp_idx(i); break;
    case S_RETURN_TYPE: s.return_type = i; break;
    case S_OCTAVES: s.octaves = i; break;
    case S_LACUNARITY: s.lacunarity = f; break;
    case S_AXIS: s.axis[vm.dim] = f; break;
    case S_VEC_SCHEME: s.vec_scheme = i; break;
    case S_POW_INT: s.pow_int = i; break;
    case S_DOMAIN_SCALE: s.dscale = f; break;
    case S_YAW: s.yaw_cos = std::cos(f); s.yaw_sin = std::sin(f); calc_rotation(s); break;   // Modifiers.h:81-83
    case S_PITCH: s.pitch_cos = std::cos(f); s.pitch_sin = std::sin(f); calc_rotation(s); break;
    case S_ROLL: s.roll_cos = std::cos(f); s.roll_sin = std::sin(f); calc_rotation(s); break;
    case S_SEED_OFFSET_NODE: s.seed_offset = i; break;
    case S_RGBA_MIN: s.rgba_min = f; break;
    case S_RGBA_MAX: s.rgba_max = f; break;
    case S_INTERP: s.interp = i; break;
    case S_CLAMP: s.clamp_output = i; break;
    case S_STEPS: s.step_count = f; s.step_recip = 1 / f; break;             // Modifiers.h:276
    case S_REMOVE_DIM: s.remove_dim = i; break;
    case S_ROT_TYPE: s.rot_type = i; break;
    default: return false;
    }
    g_epoch.fetch_add(1, std::memory_order_acq_rel);
    return true;
}

bool Node::lookup_accepts(int idx, const Node* child) const
{
    if (!child) return false;
    return !meta->lookups[idx].warp_only || is_domain_warp(child->meta->id);
}

bool Node::set_lookup(int idx, Node* child)
{
    if (idx < 0 || idx >= (int)lookups.size() || !lookup_accepts(idx, child)) return false;
    node_ref(child);
    if (lookups[idx]) node_unref(lookups[idx]);
    lookups[idx] = child;
    g_epoch.fetch_add(1, std::memory_order_acq_rel);
    return true;
}

bool Node::set_hybrid_node(int idx, Node* child)
{
    if (idx < 0 || idx >= (int)hnodes.size() || !child) return false;
    node_ref(child);
    if (hnodes[idx]) node_unref(hnodes[idx]);
    hnodes[idx] = child;
    g_epoch.fetch_add(1, std::memory_order_acq_rel);
    return true;
}

bool Node::set_hybrid_float(int idx, float v)
{
    if (idx < 0 || idx >= (int)hnodes.size()) return false;
    if (hnodes[idx]) node_unref(hnodes[idx]);
    hnodes[idx] = nullptr;                                   // HybridSource(float) drops the node link
    hvals[idx] = v;
    if (meta->id == kTerrace && v != 0.0f) st.smooth_recip = 1 + 1 / v;   // Modifiers.h:278
    g_epoch.fetch_add(1, std::memory_order_acq_rel);
    return true;
}

// ------------------------------------------------------------------ Base64

static const char kB64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

static int b64_value(unsigned char c)
{
    if (c >= 'A' && c <= 'Z') return c - 'A';
    if (c >= 'a' && c <= 'z') return c - 'a' + 26;
    if (c >= '0' && c <= '9') return c - '0' + 52;
    if (c == '+') return 62;
    if (c == '/') return 63;
    if (c == '=') return 0;
    return 64;
}

std::string base64_encode(const std::vector<uint8_t>& data)
{
    std::string plain;
    size_t n = data.size(), i = 0;
    for (; i + 2 < n; i += 3) {
        uint32_t t = (uint32_t)data[i] << 16 | (uint32_t)data[i + 1] << 8 | data[i + 2];
        plain += kB64[t >> 18 & 63]; plain += kB64[t >> 12 & 63]; plain += kB64[t >> 6 & 63]; plain += kB64[t & 63];
    }
    if (i < n) {
        uint32_t t = (uint32_t)data[i] << 16 | (i + 1 < n ? (uint32_t)data[i + 1] << 8 : 0u);
        plain += kB64[t >> 18 & 63];
        plain += kB64[t >> 12 & 63];
        plain += (i + 1 < n) ? kB64[t >> 6 & 63] : '=';
        plain += '=';
    }
    // runs of >= 3 'A' become '@' + table[run - 3]; one token covers at most 66
    std::string out;
    size_t run = 0;
    auto flush = [&]() {
        if (run >= 3) { out += '@'; out += kB64[run - 3]; }
        else out.append(run, 'A');
        run = 0;
    };
    for (char c : plain) {
        if (c == 'A') {
            if (++run == 66) flush();
        } else {
            flush();
            out += c;
        }
    }
    flush();
    return out;
}

std::vector<uint8_t> base64_decode(const char* text)
{
    if (!text) return {};
    std::string s;
    size_t raw = std::strlen(text);
    for (size_t i = 0; i < raw; ++i) {
        if (text[i] == '@') {
            if (i + 1 >= raw) return {};
            int v = b64_value((unsigned char)text[i + 1]);   // '=' counts as 0 like the reference table
            if (v >= 64) return {};
            s.append((size_t)v + 3, 'A');
            ++i;
        } else {
            s += text[i];
        }
    }
    if (s.empty() || s.size() % 4 != 0) return {};
    size_t out_len = s.size() / 4 * 3;
    if (raw >= 1 && text[raw - 1] == '=') {
        out_len--;
        if (raw >= 2 && text[raw - 2] == '=') out_len--;
    }
    std::vector<uint8_t> out;
    out.reserve(s.size() / 4 * 3);
    for (size_t k = 0; k < s.size(); k += 4) {
        uint32_t t = ((uint32_t)b64_value(s[k]) << 18) + ((uint32_t)b64_value(s[k + 1]) << 12) +
                     ((uint32_t)b64_value(s[k + 2]) << 6) + (uint32_t)b64_value(s[k + 3]);
        out.push_back((uint8_t)(t >> 16)); out.push_back((uint8_t)(t >> 8)); out.push_back((uint8_t)t);
    }
    out.resize(out_len);
    return out;
}

// ------------------------------------------------------------------ encoded trees

namespace {

enum MemberType : int { T_VAR = 0, T_LOOKUP = 1, T_HLOOKUP = 2, T_HVAR = 3, T_END = 4 };

struct Reader {
    const std::vector<uint8_t>& data;
    size_t pos = 0;
    int ends = 0;
    bool read_bytes(void* dst, size_t n)
    {
        if (ends > 0 || pos + n > data.size()) return false;
        std::memcpy(dst, data.data() + pos, n);
        pos += n;
        return true;
    }
    bool member(int& type, int& index)
    {
        if (ends > 0) { --ends; type = T_END; index = 0; return true; }
        if (pos + 1 > data.size()) return false;
        uint8_t b = data[pos++];
        type = b & 7; index = b >> 3;
        if (type == T_END) ends = index;
        return true;
    }
};

// DeserialiseSmartNodeInternal (Metadata.cpp:355-497).  Returns a node holding
// one reference owned by the caller, or nullptr.
Node* decode_node(Reader& r, std::vector<Node*>& refs)
{
    uint8_t id;
    if (!r.read_bytes(&id, 1)) return nullptr;
    if (id == 0xFF) {
        uint16_t ref;
        if (!r.read_bytes(&ref, 2) || ref >= refs.size()) return nullptr;
        node_ref(refs[ref]);
        return refs[ref];
    }
    Node* node = node_new(id);
    if (!node) return nullptr;
    auto fail = [&]() -> Node* { node_unref(node); return nullptr; };
    const NodeMeta* m = node->meta;
    int type, index;
    if (!r.member(type, index)) return fail();
    while (type == T_VAR) {
        int32_t v;
        if (!r.read_bytes(&v, 4)) return fail();
        if (index < (int)m->vars.size()) node->set_var(index, v);
        if (!r.member(type, index)) return fail();
    }
    if (type == T_LOOKUP) {
        int count = index, i = 0;
        for (; i < std::min<int>(count, (int)m->lookups.size()); ++i) {
            Node* c = decode_node(r, refs);
            bool ok = c && node->set_lookup(i, c);
            if (c) node_unref(c);
            if (!ok) return fail();
        }
        for (; i < count; ++i) {
            Node* c = decode_node(r, refs);
            if (!c) return fail();
            node_unref(c);
        }
        for (; i < (int)m->lookups.size(); ++i) {   // missing lookups get a Constant
            Node* c = node_new(kConstant);
            bool ok = node->set_lookup(i, c);
            node_unref(c);
            if (!ok) return fail();
        }
        if (!r.member(type, index)) return fail();
    }
    while (type != T_END) {
        if (type == T_HLOOKUP) {
            Node* c = decode_node(r, refs);
            if (index < (int)m->hybrids.size()) {
                bool ok = c && node->set_hybrid_node(index, c);
                if (c) node_unref(c);
                if (!ok) return fail();
            } else if (c) {
                node_unref(c);
            }
        } else if (type == T_HVAR) {
            float v;
            if (!r.read_bytes(&v, 4)) return fail();
            if (index < (int)m->hybrids.size()) node->set_hybrid_float(index, v);
        }
        if (!r.member(type, index)) return fail();
    }
    node_ref(node);           // the back-reference table holds its own reference
    refs.push_back(node);
    return node;
}

struct Writer {
    std::vector<uint8_t> out;
    int ends = 0;
    void flush_ends()
    {
        if (ends > 0) { out.push_back((uint8_t)(T_END | ((ends - 1) << 3))); ends = 0; }
    }
    void put(const void* p, size_t n)
    {
        flush_ends();
        const uint8_t* b = static_cast<const uint8_t*>(p);
        out.insert(out.end(), b, b + n);
    }
    void member(int type, int index) { uint8_t b = (uint8_t)((type & 7) | ((index & 31) << 3)); put(&b, 1); }
    void node_end() { if (++ends >= 32) flush_ends(); }
};

bool encode_node(Writer& w, const Node* n, std::unordered_map<const Node*, uint16_t>& ids)
{
    auto it = ids.find(n);
    if (it != ids.end()) {
        uint8_t ff = 0xFF;
        w.put(&ff, 1);
        w.put(&it->second, 2);
        return true;
    }
    const NodeMeta* m = n->meta;
    uint8_t id = (uint8_t)m->id;
    w.put(&id, 1);
    for (size_t i = 0; i < m->vars.size(); ++i) {
        if (n->vars[i] != m->vars[i].def) {
            w.member(T_VAR, (int)i);
            w.put(&n->vars[i], 4);
        }
    }
    if (!m->lookups.empty()) w.member(T_LOOKUP, (int)m->lookups.size());
    for (size_t i = 0; i < m->lookups.size(); ++i) {
        if (!n->lookups[i] || !encode_node(w, n->lookups[i], ids)) return false;
    }
    for (size_t i = 0; i < m->hybrids.size(); ++i) {
        if (!n->hnodes[i]) {
            if (fbits(n->hvals[i]) != fbits(m->hybrids[i].def)) {
                w.member(T_HVAR, (int)i);
                w.put(&n->hvals[i], 4);
            }
        } else {
            w.member(T_HLOOKUP, (int)i);
            if (!encode_node(w, n->hnodes[i], ids)) return false;
        }
    }
    w.node_end();
    uint16_t next = (uint16_t)ids.size();
    ids.emplace(n, next);
    return true;
}

}  // namespace

Node* decode_tree(const char* encoded)
{
    std::vector<uint8_t> data = base64_decode(encoded);
    Reader r{data};
    std::vector<Node*> refs;
    Node* root = decode_node(r, refs);
    for (Node* n : refs) node_unref(n);
    return root;
}

std::string encode_tree(const Node* root)
{
    if (!root) return "";
    Writer w;
    std::unordered_map<const Node*, uint16_t> ids;
    if (!encode_node(w, root, ids)) return "";
    w.flush_ends();
    return base64_encode(w.out);
}

}  // namespace fn
