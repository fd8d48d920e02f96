// Generator.h -- base class of the C++ node API (reference include/FastNoise/Generators/Generator.h:
// Dim, DistanceFunction, Boolean, OutputMinMax :85-105, Generator :173-450).
//
// Every node object wraps one node of libfastnoise_gb300.so and forwards to its C-ABI
// (FastNoise_C.h): the setters set members by their metadata name, and the generation calls
// run the tree on the current CUDA device.  Generation is const and may be called on one tree
// from many threads at once, as in the reference (README.md:39-40); set members before
// sharing a tree.  Output arrays of the reference-named calls are host memory; the *Device
// calls below (no reference counterpart) take device pointers and a CUDA stream.
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "../FastNoise_C.h"
#include "../Utility/Config.h"

namespace FastNoise
{
    enum class Dim
    {
        X, Y, Z, W,
        Count
    };

    constexpr static const char* kDim_Strings[] = { "X", "Y", "Z", "W" };

    enum class DistanceFunction
    {
        Euclidean,
        EuclideanSquared,
        Manhattan,
        Hybrid,
        MaxAxis,
        Minkowski,
    };

    constexpr static const char* kDistanceFunction_Strings[] =
        { "Euclidean", "Euclidean Squared", "Manhattan", "Hybrid", "Max Axis", "Minkowski" };

    enum class Boolean
    {
        False,
        True
    };

    constexpr static const char* kBoolean_Strings[] = { "False", "True" };

    static constexpr float kInfinity = std::numeric_limits<float>::infinity();

    // Smallest and largest output of a generation call.  Folding follows std::min / std::max,
    // so a NaN output never replaces a bound (Generator.h:85-105 of the reference).
    struct OutputMinMax
    {
        float min = kInfinity;
        float max = -kInfinity;

        OutputMinMax& operator <<( float v )
        {
            min = std::min( min, v );
            max = std::max( max, v );
            return *this;
        }

        OutputMinMax& operator <<( const OutputMinMax& v )
        {
            min = std::min( min, v.min );
            max = std::max( max, v.max );
            return *this;
        }
    };

    namespace Internal
    {
        struct Adopt {};                                  // construct a node object around an existing library handle

        // Metadata id of a node type by its registered name (ids follow the reference's
        // registration order, FastSIMD_Build.inl:86-143); -1 when unknown.
        inline int NodeId( const char* name )
        {
            static const std::vector<const char*> names = []
            {
                std::vector<const char*> v;
                int n = fnGetMetadataCount();
                for( int i = 0; i < n; i++ )
                {
                    v.push_back( fnGetMetadataName( i ) );
                }
                return v;
            }();
            for( size_t i = 0; i < names.size(); i++ )
            {
                if( std::strcmp( names[i], name ) == 0 )
                {
                    return (int)i;
                }
            }
            return -1;
        }

        enum MemberKind { kVariable, kNodeLookup, kHybrid };

        // Index of a member of node type `id` by name (and dimension for per-dimension
        // members), or -1.
        inline int MemberIndex( int id, MemberKind kind, const char* name, int dim )
        {
            int n = kind == kVariable ? fnGetMetadataVariableCount( id )
                  : kind == kNodeLookup ? fnGetMetadataNodeLookupCount( id ) : fnGetMetadataHybridCount( id );
            for( int i = 0; i < n; i++ )
            {
                const char* memberName = kind == kVariable ? fnGetMetadataVariableName( id, i )
                                       : kind == kNodeLookup ? fnGetMetadataNodeLookupName( id, i ) : fnGetMetadataHybridName( id, i );
                int memberDim = kind == kVariable ? fnGetMetadataVariableDimensionIdx( id, i )
                              : kind == kNodeLookup ? fnGetMetadataNodeLookupDimensionIdx( id, i ) : fnGetMetadataHybridDimensionIdx( id, i );
                if( memberDim == dim && std::strcmp( memberName, name ) == 0 )
                {
                    return i;
                }
            }
            return -1;
        }
    }

    class Generator
    {
    public:
        Generator( const Generator& ) = delete;
        Generator( Generator&& ) = delete;

        virtual ~Generator()
        {
            fnDeleteNodeRef( mNode );
        }

        FastSIMD::FeatureSet GetActiveFeatureSet() const
        {
            return static_cast<FastSIMD::FeatureSet>( fnGetActiveFeatureSet( mNode ) );
        }

        // The node type's metadata (defined in Metadata.h)
        const Metadata& GetMetadata() const;

        // ---- generation into host memory: the reference's calls (Generator.h:210-429) ----

        OutputMinMax GenUniformGrid2D( float* out,
            float xOffset, float yOffset,
            int xCount, int yCount,
            float xStepSize, float yStepSize,
            int seed ) const
        {
            float mm[2];
            fnGenUniformGrid2D( mNode, out, xOffset, yOffset, xCount, yCount, xStepSize, yStepSize, seed, mm );
            return Result( mm );
        }

        OutputMinMax GenUniformGrid3D( float* out,
            float xOffset, float yOffset, float zOffset,
            int xCount, int yCount, int zCount,
            float xStepSize, float yStepSize, float zStepSize,
            int seed ) const
        {
            float mm[2];
            fnGenUniformGrid3D( mNode, out, xOffset, yOffset, zOffset, xCount, yCount, zCount, xStepSize, yStepSize, zStepSize,
                                seed, mm );
            return Result( mm );
        }

        OutputMinMax GenUniformGrid4D( float* out,
            float xOffset, float yOffset, float zOffset, float wOffset,
            int xCount, int yCount, int zCount, int wCount,
            float xStepSize, float yStepSize, float zStepSize, float wStepSize,
            int seed ) const
        {
            float mm[2];
            fnGenUniformGrid4D( mNode, out, xOffset, yOffset, zOffset, wOffset, xCount, yCount, zCount, wCount, xStepSize,
                                yStepSize, zStepSize, wStepSize, seed, mm );
            return Result( mm );
        }

        OutputMinMax GenTileable2D( float* out,
            int xSize, int ySize,
            float xStepSize, float yStepSize,
            int seed ) const
        {
            float mm[2];
            fnGenTileable2D( mNode, out, xSize, ySize, xStepSize, yStepSize, seed, mm );
            return Result( mm );
        }

        OutputMinMax GenPositionArray2D( float* out, int count,
            const float* xPosArray, const float* yPosArray,
            float xOffset, float yOffset, int seed ) const
        {
            float mm[2];
            fnGenPositionArray2D( mNode, out, count, xPosArray, yPosArray, xOffset, yOffset, seed, mm );
            return Result( mm );
        }

        OutputMinMax GenPositionArray3D( float* out, int count,
            const float* xPosArray, const float* yPosArray, const float* zPosArray,
            float xOffset, float yOffset, float zOffset, int seed ) const
        {
            float mm[2];
            fnGenPositionArray3D( mNode, out, count, xPosArray, yPosArray, zPosArray, xOffset, yOffset, zOffset, seed, mm );
            return Result( mm );
        }

        OutputMinMax GenPositionArray4D( float* out, int count,
            const float* xPosArray, const float* yPosArray, const float* zPosArray, const float* wPosArray,
            float xOffset, float yOffset, float zOffset, float wOffset, int seed ) const
        {
            float mm[2];
            fnGenPositionArray4D( mNode, out, count, xPosArray, yPosArray, zPosArray, wPosArray, xOffset, yOffset, zOffset,
                                  wOffset, seed, mm );
            return Result( mm );
        }

        float GenSingle2D( float x, float y, int seed ) const { return fnGenSingle2D( mNode, x, y, seed ); }
        float GenSingle3D( float x, float y, float z, int seed ) const { return fnGenSingle3D( mNode, x, y, z, seed ); }
        float GenSingle4D( float x, float y, float z, float w, int seed ) const { return fnGenSingle4D( mNode, x, y, z, w, seed ); }

        // ---- generation into device memory (no reference counterpart) ----
        // dOut: device array; dMinMax: NULL or device float[2]; stream: a cudaStream_t (NULL =
        // the legacy default stream).  Asynchronous; returns FN_OK or a negative FN_ERR_* status.

        int GenUniformGrid2DDevice( float* dOut, float xOffset, float yOffset, int xCount, int yCount,
            float xStepSize, float yStepSize, int seed, float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenUniformGrid2DDevice( mNode, dOut, xOffset, yOffset, xCount, yCount, xStepSize, yStepSize, seed,
                                             dMinMax, stream );
        }

        int GenUniformGrid3DDevice( float* dOut, float xOffset, float yOffset, float zOffset,
            int xCount, int yCount, int zCount, float xStepSize, float yStepSize, float zStepSize,
            int seed, float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenUniformGrid3DDevice( mNode, dOut, xOffset, yOffset, zOffset, xCount, yCount, zCount, xStepSize,
                                             yStepSize, zStepSize, seed, dMinMax, stream );
        }

        int GenUniformGrid4DDevice( float* dOut, float xOffset, float yOffset, float zOffset, float wOffset,
            int xCount, int yCount, int zCount, int wCount,
            float xStepSize, float yStepSize, float zStepSize, float wStepSize,
            int seed, float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenUniformGrid4DDevice( mNode, dOut, xOffset, yOffset, zOffset, wOffset, xCount, yCount, zCount, wCount,
                                             xStepSize, yStepSize, zStepSize, wStepSize, seed, dMinMax, stream );
        }

        int GenTileable2DDevice( float* dOut, int xSize, int ySize, float xStepSize, float yStepSize,
            int seed, float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenTileable2DDevice( mNode, dOut, xSize, ySize, xStepSize, yStepSize, seed, dMinMax, stream );
        }

        int GenPositionArray2DDevice( float* dOut, int count, const float* dX, const float* dY,
            float xOffset, float yOffset, int seed, float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenPositionArray2DDevice( mNode, dOut, count, dX, dY, xOffset, yOffset, seed, dMinMax, stream );
        }

        int GenPositionArray3DDevice( float* dOut, int count, const float* dX, const float* dY, const float* dZ,
            float xOffset, float yOffset, float zOffset, int seed, float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenPositionArray3DDevice( mNode, dOut, count, dX, dY, dZ, xOffset, yOffset, zOffset, seed, dMinMax,
                                               stream );
        }

        int GenPositionArray4DDevice( float* dOut, int count, const float* dX, const float* dY, const float* dZ,
            const float* dW, float xOffset, float yOffset, float zOffset, float wOffset, int seed,
            float* dMinMax = nullptr, void* stream = nullptr ) const
        {
            return fnGenPositionArray4DDevice( mNode, dOut, count, dX, dY, dZ, dW, xOffset, yOffset, zOffset, wOffset, seed,
                                               dMinMax, stream );
        }

        // The library handle this object wraps, for mixing with C-ABI calls (batches, the
        // request server, fnJitCompile).  The object keeps its reference; take your own with
        // the node's lifetime in mind.
        void* GetNodeHandle() const noexcept { return mNode; }

    protected:
        // Only intermediate classes name this; the most-derived class always picks one below.
        Generator() noexcept : mNode( nullptr ) {}

        // A new node of metadata type `id` (its reference defaults).
        explicit Generator( int id ) : mNode( id >= 0 ? fnNewFromMetadata( id, 0 ) : nullptr ) {}

        // Take over one reference to an existing node.
        Generator( Internal::Adopt, void* node ) noexcept : mNode( node ) {}

        // Member setters by metadata name; false when the node has no such member or the
        // library refuses the value (a source of the wrong type).
        bool SetVariable( const char* name, float value, int dim = -1 )
        {
            int i = Internal::MemberIndex( fnGetMetadataID( mNode ), Internal::kVariable, name, dim );
            return i >= 0 && fnSetVariableFloat( mNode, i, value );
        }

        bool SetVariable( const char* name, int value, int dim = -1 )
        {
            int i = Internal::MemberIndex( fnGetMetadataID( mNode ), Internal::kVariable, name, dim );
            return i >= 0 && fnSetVariableIntEnum( mNode, i, value );
        }

        bool SetNodeLookup( const char* name, SmartNodeArg<> gen, int dim = -1 )
        {
            int i = Internal::MemberIndex( fnGetMetadataID( mNode ), Internal::kNodeLookup, name, dim );
            return i >= 0 && gen && fnSetNodeLookup( mNode, i, gen->GetNodeHandle() );
        }

        bool SetHybrid( const char* name, SmartNodeArg<> gen, int dim = -1 )
        {
            int i = Internal::MemberIndex( fnGetMetadataID( mNode ), Internal::kHybrid, name, dim );
            return i >= 0 && gen && fnSetHybridNodeLookup( mNode, i, gen->GetNodeHandle() );
        }

        bool SetHybrid( const char* name, float value, int dim = -1 )
        {
            int i = Internal::MemberIndex( fnGetMetadataID( mNode ), Internal::kHybrid, name, dim );
            return i >= 0 && fnSetHybridFloat( mNode, i, value );
        }

    private:
        template<typename>
        friend class SmartNode;

        static OutputMinMax Result( const float* mm )
        {
            OutputMinMax r;
            r.min = mm[0];
            r.max = mm[1];
            return r;
        }

        // Adds `add` to the object's reference count and returns the count before.
        int32_t RefAdd( int32_t add ) const noexcept
        {
            return mRefs.fetch_add( add, std::memory_order_acq_rel );
        }

        void* mNode;
        mutable std::atomic<int32_t> mRefs{ 0 };
    };
}

// Declares a concrete node class's constructors and its type name.
#define FASTNOISE_GB300_NODE( CLASS )                                                        \
public:                                                                                      \
    using FastNoiseConcreteType = CLASS;                                                     \
    static const char* MetadataName() { return #CLASS; }                                     \
    CLASS() : ::FastNoise::Generator( ::FastNoise::Internal::NodeId( #CLASS ) ) {}           \
    CLASS( ::FastNoise::Internal::Adopt a, void* node ) : ::FastNoise::Generator( a, node ) {}

#include "../Metadata.h"
