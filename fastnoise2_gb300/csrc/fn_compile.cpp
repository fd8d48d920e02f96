// fn_compile.cpp -- node tree -> device program.
//
// The compiler walks the tree exactly like the reference's recursive Gen calls
// (include/FastNoise/Generators/*.inl) and emits one instruction per node
// operation.  Seeds are tracked symbolically as "call seed + immediate" (every
// seed change in the reference is a constant add: Seeded offsets, fractal
// octaves, SeedOffset, CellularLookup's +1), so no seed registers exist.
// Positions are groups of `dim` consecutive registers.
#include "fn_compile.h"

#include <cstddef>
#include <cstring>

namespace fn {

uint64_t fnv1a64(const void* data, size_t n, uint64_t h)
{
    const uint8_t* p = static_cast<const uint8_t*>(data);
    for (size_t i = 0; i < n; ++i) { h ^= p[i]; h *= 1099511628211ull; }
    return h;
}

namespace {

constexpr float kValueBounds = 2147483648.f;
constexpr float kJitter[5] = {0, 0, 0.437016f, 0.396144f, 0.366025f};   // Cellular.inl:11-13

// Native output bounds of the coherent noise kernels (Simplex.inl:60,139,283,
// :374,574,933; Perlin.inl:32,71,122; Value uses kValueBounds).
float noise_bound(int kind, int dim)
{
    switch (kind) {
    case FN_NOISE_SIMPLEX:
        return dim == 2 ? 0.0261208079755306243896484375f : dim == 3 ? 0.030586399137973785400390625f : 0.036730043590068817138671875f;
    case FN_NOISE_SUPERSIMPLEX:
        return dim == 2 ? 0.14084912836551666259765625f : dim == 3 ? 0.0069091119803488254547119140625f : 0.011310013942420482635498046875f;
    case FN_NOISE_PERLIN:
        return dim == 2 ? 1.726796627044677734375f : dim == 3 ? (float)1.0363423824310302734375 : 1.33858621120452880859375f;
    default:
        return kValueBounds;
    }
}

// VariableRange::ScaleOutput multiplier (BasicGenerators.inl:29)
float range_mul(const NodeState& st, float nmin, float nmax) { return (1.0f / (nmax - nmin)) * st.range_scale; }

class Compiler {
public:
    std::vector<FnInstr> code;
    std::vector<float> params;
    std::vector<CompiledProgram> subs;   // per-cell sub-programs (node-driven Minkowski P)
    std::string err;
    int max_reg = -1;
    uint64_t used = 0;     // bit r set = register r holds a live value

    bool ok() const { return err.empty(); }

    int alloc(int n)
    {
        for (int base = 0; base + n <= FN_MAX_REGS; ++base) {
            bool free = true;
            for (int k = 0; k < n && free; ++k) free = !(used >> (base + k) & 1ull);
            if (free) {
                for (int k = 0; k < n; ++k) used |= 1ull << (base + k);
                if (base + n - 1 > max_reg) max_reg = base + n - 1;
                return base;
            }
        }
        fail("tree needs more than 64 live registers");
        return 0;
    }
    void release(int base, int n)
    {
        for (int k = 0; k < n; ++k) used &= ~(1ull << (base + k));
    }
    void fail(const std::string& e) { if (err.empty()) err = e; }

    int param(float v) { params.push_back(v); return (int)params.size() - 1; }
    int param_block(std::initializer_list<float> vs)
    {
        int at = (int)params.size();
        params.insert(params.end(), vs.begin(), vs.end());
        return at;
    }

    void emit(FnOp op, int dim, int dst, int a = FN_REG_NONE, int b = FN_REG_NONE, int c = FN_REG_NONE, int d = FN_REG_NONE,
              int e = FN_REG_NONE, int prm = 0, int aux = 0, int32_t seed = 0)
    {
        if (code.size() >= FN_MAX_INSTR) { fail("program exceeds instruction limit"); return; }
        if (prm >= 65536) { fail("program exceeds parameter limit"); return; }
        FnInstr in;
        in.op = (uint8_t)op; in.dim = (uint8_t)dim; in.dst = (uint8_t)dst; in.a = (uint8_t)a;
        in.b = (uint8_t)b; in.c = (uint8_t)c; in.d = (uint8_t)d; in.e = (uint8_t)e;
        in.prm = (uint16_t)prm; in.aux = (uint16_t)aux; in.seed = seed;
        code.push_back(in);
    }

    int constant(float v)
    {
        int r = alloc(1);
        emit(FN_OP_CONST, 1, r, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, param(v));
        return r;
    }

    // HybridSource: node value at (pos, seed) or the constant (Generator.inl:48-58)
    int hybrid(const Node* n, int k, int dim, int32_t seed, int pos)
    {
        if (n->hnodes[k]) return gen(n->hnodes[k], dim, seed, pos);
        return constant(n->hvals[k]);
    }

    int copy_pos(int pos, int dim)
    {
        int q = alloc(dim);
        for (int k = 0; k < dim; ++k) emit(FN_OP_MOV, 1, q + k, pos + k);
        return q;
    }

    int lookup(const Node* n, int k)
    {
        if (!n->lookups[k]) { fail(std::string(n->meta->name) + ": source '" + n->meta->lookups[k].name + "' is not set"); return -1; }
        return k;
    }

    static int32_t sadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

    // Warp instruction of a domain-warp node: lattice gradient, or simplex /
    // super-simplex with the node's vectorization scheme (DomainWarpSimplex.h).
    static FnOp warp_op(const Node* w) { return w->meta->id == kDomainWarpGradient ? FN_OP_WARP_GRAD : FN_OP_WARP_SIMPLEX; }
    static uint16_t warp_aux(const Node* w)
    {
        if (w->meta->id == kDomainWarpGradient) return 0;
        return (uint16_t)((w->meta->id == kDomainWarpSuperSimplex ? 1 : 0) | (w->st.vec_scheme == 1 ? 2 : 0));
    }

    int gen(const Node* n, int dim, int32_t seed, int pos);
    static bool compile_sub(const Node* root, int dim, int32_t seed, CompiledProgram& out, std::string& error);
};

int Compiler::gen(const Node* n, int dim, int32_t seed, int pos)
{
    if (!ok()) return 0;
    const NodeState& s = n->st;
    const int id = n->meta->id;
    switch (id) {
    case kConstant:
        return constant(s.value);

    case kSimplex: case kSuperSimplex: case kPerlin: case kValue: {
        int kind = id == kSimplex ? FN_NOISE_SIMPLEX : id == kSuperSimplex ? FN_NOISE_SUPERSIMPLEX : id == kPerlin ? FN_NOISE_PERLIN : FN_NOISE_VALUE;
        float b = noise_bound(kind, dim);
        int r = alloc(1);
        int prm = param_block({s.frequency, -b, range_mul(s, -b, b), s.range_min});
        emit(FN_OP_NOISE, dim, r, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, prm, kind, sadd(seed, s.seed_offset));
        return r;
    }
    case kWhite: {
        int r = alloc(1);
        int prm = param_block({range_mul(s, -kValueBounds, kValueBounds), s.range_min});
        emit(FN_OP_WHITE, dim, r, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, prm, 0, sadd(seed, s.seed_offset));
        return r;
    }
    case kCheckerboard: {
        int r = alloc(1);
        emit(FN_OP_CHECKER, dim, r, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE,
             param_block({s.frequency, range_mul(s, 0, 2), s.range_min}));
        return r;
    }
    case kSineWave: {
        int r = alloc(1);
        emit(FN_OP_SINE, dim, r, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE,
             param_block({s.frequency, range_mul(s, -1, 1), s.range_min}));
        return r;
    }
    case kGradient: {
        int off[4] = {FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE};
        for (int k = 0; k < dim; ++k) off[k] = hybrid(n, k, dim, seed, pos);
        int r = alloc(1);
        emit(FN_OP_GRADIENT, dim, r, pos, off[0], off[1], off[2], off[3],
             param_block({s.multiplier[0], s.multiplier[1], s.multiplier[2], s.multiplier[3]}));
        for (int k = 0; k < dim; ++k) release(off[k], 1);
        return r;
    }
    case kDistanceToPoint: {
        int pt[4] = {FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE};
        for (int k = 0; k < dim; ++k) pt[k] = hybrid(n, k, dim, seed, pos);
        int d = alloc(dim);
        emit(FN_OP_SUB_POS, dim, d, pos, pt[0], pt[1], pt[2], pt[3]);
        for (int k = 0; k < dim; ++k) release(pt[k], 1);
        int mk = FN_REG_NONE;
        if (s.dist_func == 5) mk = hybrid(n, 4, dim, seed, d);    // Minkowski P sampled at the offset vector
        int r = alloc(1);
        const int df = (s.dist_func < 0 || s.dist_func > 5) ? 0 : s.dist_func;   // switch default: Euclidean
        emit(FN_OP_DISTANCE, dim, r, d, mk, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, 0, df | (1 << 4));
        if (mk != FN_REG_NONE) release(mk, 1);
        release(d, dim);
        return r;
    }
    case kCellularValue: case kCellularDistance: case kCellularLookup: {
        // Cellular.inl:22-30: jitters sampled at the unscaled position with the incoming seed
        int jit = hybrid(n, 1, dim, seed, pos);
        bool size_active = n->hnodes[2] != nullptr || n->hvals[2] != 0.0f;
        int sj = size_active ? hybrid(n, 2, dim, seed, pos) : FN_REG_NONE;
        const int32_t cell_seed = sadd(seed, s.seed_offset);
        int df = (s.dist_func < 0 || s.dist_func > 5) ? 0 : s.dist_func;
        // Minkowski P driven by a node: a sub-program evaluated at every cell's offset
        // vector with the incoming seed (Cellular.inl:63, Utils.inl:326-331)
        int sub = FN_REG_NONE;
        if (df == 5 && n->hnodes[0]) {
            if (subs.size() >= 255) { fail("too many per-cell sub-programs"); return 0; }
            CompiledProgram sp;
            std::string e;
            if (!compile_sub(n->hnodes[0], dim, seed, sp, e)) { fail(e); return 0; }
            sub = (int)subs.size();
            subs.push_back(std::move(sp));
        }
        if (id == kCellularValue) {
            int r = alloc(1);
            int prm = param_block({s.frequency, range_mul(s, -kValueBounds, kValueBounds), s.range_min, n->hvals[0]});
            emit(FN_OP_CELL_VALUE, dim, r, pos, jit, sj, sub, FN_REG_NONE, prm, df | (s.value_index << 4), cell_seed);
            release(jit, 1); if (sj != FN_REG_NONE) release(sj, 1);
            return r;
        }
        if (id == kCellularDistance) {
            // CellularDistance::GetReturn native max (Cellular.inl:531-565)
            float maxDist = 1 + kJitter[dim];
            maxDist *= maxDist;
            int ret = (s.return_type < 0 || s.return_type > 4) ? 0 : s.return_type;
            float nmax = ret == 1 ? maxDist * 2 : ret == 3 ? maxDist * maxDist : maxDist;
            int r = alloc(1);
            int prm = param_block({s.frequency, range_mul(s, 0, nmax), s.range_min, n->hvals[0]});
            emit(FN_OP_CELL_DIST, dim, r, pos, jit, sj, sub, FN_REG_NONE, prm,
                 df | (s.dist_idx0 << 4) | (s.dist_idx1 << 8) | (ret << 12), cell_seed);
            release(jit, 1); if (sj != FN_REG_NONE) release(sj, 1);
            return r;
        }
        if (lookup(n, 0) < 0) return 0;
        int q = alloc(dim);
        emit(FN_OP_CELL_LOOKUP, dim, q, pos, jit, sj, sub, FN_REG_NONE, param_block({s.frequency, s.scale, n->hvals[0]}), df, cell_seed);
        release(jit, 1); if (sj != FN_REG_NONE) release(sj, 1);
        int r = gen(n->lookups[0], dim, sadd(seed, 1), q);      // Cellular.inl:633 (sourceSeed - (-1))
        release(q, dim);
        return r;
    }

    case kFractalFBm: case kFractalRidged: {
        if (lookup(n, 0) < 0) return 0;
        const int ridged = id == kFractalRidged;
        int gain = hybrid(n, 0, dim, seed, pos);
        int ws = hybrid(n, 1, dim, seed, pos);
        int noise = gen(n->lookups[0], dim, seed, pos);
        int sum = alloc(1), amp = alloc(1);
        emit(FN_OP_FRACT_INIT, dim, sum, noise, amp, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, 0, ridged);
        int p = pos;
        int32_t sd = seed;
        for (int i = 1; i < s.octaves; ++i) {
            sd = sadd(sd, 1);
            emit(FN_OP_FRACT_AMP, dim, amp, noise, amp, ws, gain, FN_REG_NONE, 0, ridged);
            int q = alloc(dim);
            emit(FN_OP_SCALE_POS, dim, q, p, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, param(s.lacunarity));
            if (p != pos) release(p, dim);
            p = q;
            release(noise, 1);
            noise = gen(n->lookups[0], dim, sd, p);
            emit(FN_OP_FRACT_ACC, dim, sum, noise, amp, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, 0, ridged);
            if (!ok()) return 0;
        }
        if (p != pos) release(p, dim);
        release(noise, 1); release(amp, 1); release(gain, 1); release(ws, 1);
        return sum;
    }

    case kPingPong: {
        if (lookup(n, 0) < 0) return 0;
        int st_ = hybrid(n, 0, dim, seed, pos);
        int v = gen(n->lookups[0], dim, seed, pos);
        int r = alloc(1);
        emit(FN_OP_PINGPONG, dim, r, v, st_);
        release(v, 1); release(st_, 1);
        return r;
    }

    case kDomainWarpGradient: case kDomainWarpSimplex: case kDomainWarpSuperSimplex: {
        // DomainWarp::GenT (DomainWarp.inl:9-17): seed offset applied in GenT and again in Warp
        if (lookup(n, 0) < 0) return 0;
        int amp = hybrid(n, 0, dim, seed, pos);
        int w = copy_pos(pos, dim);
        emit(warp_op(n), dim, w, pos, amp, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE,
             param_block({s.frequency, s.axis[0], s.axis[1], s.axis[2], s.axis[3]}), warp_aux(n),
             sadd(sadd(seed, s.seed_offset), s.seed_offset));
        release(amp, 1);
        int r = gen(n->lookups[0], dim, seed, w);
        release(w, dim);
        return r;
    }

    case kDomainWarpFractalProgressive: case kDomainWarpFractalIndependent: {
        // DomainWarpFractal.inl:9-73
        if (lookup(n, 0) < 0) return 0;
        const Node* warp = n->lookups[0];
        if (!warp->lookups[0]) { fail(std::string(warp->meta->name) + ": source is not set"); return 0; }
        const bool indep = id == kDomainWarpFractalIndependent;
        const NodeState& ws_ = warp->st;
        int amp = hybrid(warp, 0, dim, seed, pos);
        int wstr = hybrid(n, 1, dim, seed, pos);
        int gain = hybrid(n, 0, dim, seed, pos);
        int w = copy_pos(pos, dim);
        int strength = alloc(1);
        float freq = ws_.frequency;
        const int src = indep ? pos : w;
        emit(warp_op(warp), dim, w, src, amp, strength, FN_REG_NONE, FN_REG_NONE,
             param_block({freq, ws_.axis[0], ws_.axis[1], ws_.axis[2], ws_.axis[3]}), warp_aux(warp), sadd(seed, ws_.seed_offset));
        int32_t sd = seed;
        for (int i = 1; i < s.octaves; ++i) {
            sd = sadd(sd, 1);
            freq = freq * s.lacunarity;
            emit(FN_OP_DWF_AMP, dim, amp, strength, amp, wstr, gain);
            emit(warp_op(warp), dim, w, src, amp, strength, FN_REG_NONE, FN_REG_NONE,
                 param_block({freq, ws_.axis[0], ws_.axis[1], ws_.axis[2], ws_.axis[3]}), warp_aux(warp), sadd(sd, ws_.seed_offset));
        }
        release(amp, 1); release(wstr, 1); release(gain, 1); release(strength, 1);
        int r = gen(warp->lookups[0], dim, seed, w);
        release(w, dim);
        return r;
    }

    case kAdd: case kMultiply: case kMin: case kMax: {
        if (lookup(n, 0) < 0) return 0;
        int l = gen(n->lookups[0], dim, seed, pos);
        int rr = hybrid(n, 0, dim, seed, pos);
        int r = alloc(1);
        FnOp op = id == kAdd ? FN_OP_ADD : id == kMultiply ? FN_OP_MUL : id == kMin ? FN_OP_MIN : FN_OP_MAX;
        emit(op, dim, r, l, rr);
        release(l, 1); release(rr, 1);
        return r;
    }
    case kSubtract: case kDivide: case kModulus: case kPowFloat: {
        int l = hybrid(n, 0, dim, seed, pos);
        int rr = hybrid(n, 1, dim, seed, pos);
        int r = alloc(1);
        FnOp op = id == kSubtract ? FN_OP_SUB : id == kDivide ? FN_OP_DIV : id == kModulus ? FN_OP_MOD : FN_OP_POWF;
        emit(op, dim, r, l, rr);
        release(l, 1); release(rr, 1);
        return r;
    }
    case kMinSmooth: case kMaxSmooth: {
        if (lookup(n, 0) < 0) return 0;
        int l = gen(n->lookups[0], dim, seed, pos);
        int rr = hybrid(n, 0, dim, seed, pos);
        int sm = hybrid(n, 1, dim, seed, pos);
        int r = alloc(1);
        emit(id == kMinSmooth ? FN_OP_MINSMOOTH : FN_OP_MAXSMOOTH, dim, r, l, rr, sm);
        release(l, 1); release(rr, 1); release(sm, 1);
        return r;
    }
    case kAbs: case kSignedSquareRoot: case kPowInt: case kConvertRGBA8: {
        if (lookup(n, 0) < 0) return 0;
        int v = gen(n->lookups[0], dim, seed, pos);
        int r = alloc(1);
        if (id == kAbs) emit(FN_OP_ABS, dim, r, v);
        else if (id == kSignedSquareRoot) emit(FN_OP_SSQRT, dim, r, v);
        else if (id == kPowInt) emit(FN_OP_POWI, dim, r, v, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, 0, s.pow_int < 2 ? 2 : (s.pow_int > 65535 ? 65535 : s.pow_int));
        else emit(FN_OP_RGBA8, dim, r, v, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, param_block({s.rgba_min, s.rgba_max}));
        release(v, 1);
        return r;
    }

    case kDomainScale: case kDomainAxisScale: {
        if (lookup(n, 0) < 0) return 0;
        int q = alloc(dim);
        if (id == kDomainScale) emit(FN_OP_SCALE_POS, dim, q, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, param(s.dscale));
        else emit(FN_OP_SCALE_POS_V, dim, q, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, param_block({s.axis[0], s.axis[1], s.axis[2], s.axis[3]}));
        int r = gen(n->lookups[0], dim, seed, q);
        release(q, dim);
        return r;
    }
    case kDomainOffset: {
        if (lookup(n, 0) < 0) return 0;
        int off[4] = {FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE};
        for (int k = 0; k < dim; ++k) off[k] = hybrid(n, k, dim, seed, pos);
        int q = alloc(dim);
        emit(FN_OP_OFFSET_POS, dim, q, pos, off[0], off[1], off[2], off[3]);
        for (int k = 0; k < dim; ++k) release(off[k], 1);
        int r = gen(n->lookups[0], dim, seed, q);
        release(q, dim);
        return r;
    }
    case kDomainRotate: {   // Modifiers.inl:33-61
        if (lookup(n, 0) < 0) return 0;
        if (dim == 4) return gen(n->lookups[0], 4, seed, pos);
        if (dim == 2 && s.pitch_sin == 0.0f && s.roll_sin == 0.0f) {
            int q = alloc(2);
            emit(FN_OP_ROTATE2, 2, q, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, param_block({s.yaw_cos, s.yaw_sin}));
            int r = gen(n->lookups[0], 2, seed, q);
            release(q, 2);
            return r;
        }
        int q = alloc(3);
        emit(FN_OP_ROTATE3, dim, q, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE,
             param_block({s.rot[0], s.rot[1], s.rot[2], s.rot[3], s.rot[4], s.rot[5], s.rot[6], s.rot[7], s.rot[8]}));
        int r = gen(n->lookups[0], 3, seed, q);
        release(q, 3);
        return r;
    }
    case kDomainRotatePlane: {   // Modifiers.inl:354-408
        if (lookup(n, 0) < 0) return 0;
        int od = dim == 2 ? 3 : dim;
        int q = alloc(od);
        emit(FN_OP_ROTPLANE, dim, q, pos, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE, 0, dim == 2 ? 0 : s.rot_type);
        int r = gen(n->lookups[0], od, seed, q);
        release(q, od);
        return r;
    }
    case kSeedOffset:
        if (lookup(n, 0) < 0) return 0;
        return gen(n->lookups[0], dim, sadd(seed, s.seed_offset), pos);
    case kGeneratorCache:
        if (lookup(n, 0) < 0) return 0;
        return gen(n->lookups[0], dim, seed, pos);

    case kFade: {
        if (lookup(n, 0) < 0 || lookup(n, 1) < 0) return 0;
        int f = hybrid(n, 0, dim, seed, pos), fmn = hybrid(n, 1, dim, seed, pos), fmx = hybrid(n, 2, dim, seed, pos);
        int a = gen(n->lookups[0], dim, seed, pos);
        int b = gen(n->lookups[1], dim, seed, pos);
        int r = alloc(1);
        emit(FN_OP_FADE, dim, r, a, b, f, fmn, fmx, 0, s.interp);
        release(a, 1); release(b, 1); release(f, 1); release(fmn, 1); release(fmx, 1);
        return r;
    }
    case kRemap: {
        if (lookup(n, 0) < 0) return 0;
        int v = gen(n->lookups[0], dim, seed, pos);
        int h[4];
        for (int k = 0; k < 4; ++k) h[k] = hybrid(n, k, dim, seed, pos);
        int r = alloc(1);
        emit(FN_OP_REMAP, dim, r, v, h[0], h[1], h[2], h[3], 0, s.clamp_output == 1);
        release(v, 1);
        for (int k = 0; k < 4; ++k) release(h[k], 1);
        return r;
    }
    case kTerrace: {
        if (lookup(n, 0) < 0) return 0;
        int v = gen(n->lookups[0], dim, seed, pos);
        int sm = n->hnodes[0] ? gen(n->hnodes[0], dim, seed, pos) : FN_REG_NONE;
        int r = alloc(1);
        emit(FN_OP_TERRACE, dim, r, v, sm, FN_REG_NONE, FN_REG_NONE, FN_REG_NONE,
             param_block({s.step_count, s.step_recip, s.smooth_recip}), (!n->hnodes[0] && n->hvals[0] != 0.0f) ? 1 : 0);
        release(v, 1);
        if (sm != FN_REG_NONE) release(sm, 1);
        return r;
    }
    case kAddDimension: {
        if (lookup(n, 0) < 0) return 0;
        if (dim == 4) return gen(n->lookups[0], 4, seed, pos);
        int nd = hybrid(n, 0, dim, seed, pos);
        int q = alloc(dim + 1);
        for (int k = 0; k < dim; ++k) emit(FN_OP_MOV, 1, q + k, pos + k);
        emit(FN_OP_MOV, 1, q + dim, nd);
        release(nd, 1);
        int r = gen(n->lookups[0], dim + 1, seed, q);
        release(q, dim + 1);
        return r;
    }
    case kRemoveDimension: {   // Modifiers.inl:240-275
        if (lookup(n, 0) < 0) return 0;
        int rm = s.remove_dim;
        if (dim == 2 || rm < 0 || rm >= dim) return gen(n->lookups[0], dim, seed, pos);
        int q = alloc(dim - 1), m = 0;
        for (int k = 0; k < dim; ++k)
            if (k != rm) emit(FN_OP_MOV, 1, q + m++, pos + k);
        int r = gen(n->lookups[0], dim - 1, seed, q);
        release(q, dim - 1);
        return r;
    }
    default:
        fail(std::string("unknown node id ") + std::to_string(id));
        return 0;
    }
}

}  // namespace

namespace {

// Serialise a finished compiler into a program blob (fn_program.h) and hash it.
bool finalize(Compiler& c, int dim, int out_reg, CompiledProgram& out, std::string& error)
{
    FnProgramHeader h;
    std::memset(&h, 0, sizeof h);
    h.magic = FN_PROGRAM_MAGIC;
    h.n_instr = (uint16_t)c.code.size();
    h.n_regs = (uint16_t)(c.max_reg + 1);
    h.n_params = (uint16_t)c.params.size();
    h.dim = (uint8_t)dim;
    h.out_reg = (uint8_t)out_reg;
    h.flags = c.subs.empty() ? 0u : 1u;
    if (c.params.size() > FN_MAX_PARAMS) { error = "program exceeds parameter limit"; return false; }
    size_t bytes = sizeof(h) + c.code.size() * sizeof(FnInstr) + c.params.size() * sizeof(float);
    bytes = (bytes + 15) & ~(size_t)15;
    h.bytes = (uint32_t)bytes;
    out.blob.assign(bytes, 0);
    std::memcpy(out.blob.data() + sizeof(h), c.code.data(), c.code.size() * sizeof(FnInstr));
    std::memcpy(out.blob.data() + sizeof(h) + c.code.size() * sizeof(FnInstr), c.params.data(), c.params.size() * sizeof(float));
    uint64_t hash = fnv1a64(out.blob.data() + sizeof(h), bytes - sizeof(h), fnv1a64(&h, offsetof(FnProgramHeader, flags)));
    for (const auto& sp : c.subs) hash = fnv1a64(&sp.hash, sizeof sp.hash, hash);
    h.hash = hash;
    std::memcpy(out.blob.data(), &h, sizeof(h));
    out.hash = h.hash;
    out.dim = dim;
    out.n_instr = h.n_instr;
    out.n_regs = h.n_regs;
    out.subs = std::move(c.subs);
    return true;
}

}  // namespace

bool Compiler::compile_sub(const Node* root, int dim, int32_t seed, CompiledProgram& out, std::string& error)
{
    Compiler c;
    int pos = c.alloc(dim);                 // the cell's offset vector: registers 0 .. dim-1
    int r = c.gen(root, dim, seed, pos);
    if (!c.ok()) { error = c.err; return false; }
    return finalize(c, dim, r, out, error);
}

bool compile_program(const Node* root, int dim, CompiledProgram& out, std::string& error)
{
    if (!root) { error = "null node"; return false; }
    if (dim < 2 || dim > 4) { error = "dimension must be 2, 3 or 4"; return false; }
    Compiler c;
    int pos = c.alloc(dim);                 // root position: registers 0 .. dim-1
    int r = c.gen(root, dim, 0, pos);
    if (!c.ok()) { error = c.err; return false; }
    return finalize(c, dim, r, out, error);
}

}  // namespace fn
