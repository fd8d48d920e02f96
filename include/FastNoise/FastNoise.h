// FastNoise.h -- the C++ node API of the GB300 backend (reference include/FastNoise/FastNoise.h:
// New<T> :36-43, NewFromEncodedNodeTree :65).
//
// Header-only C++ over the C-ABI of libfastnoise_gb300.so (link with -lfastnoise_gb300): the
// node classes, SmartNode, Metadata and the Generator calls returning OutputMinMax keep the
// reference's names and signatures, so C++ code written against FastNoise2 compiles unchanged
// and its trees run on the current CUDA device.
#pragma once
#include "Utility/Config.h"

#include "Generators/BasicGenerators.h"
#include "Generators/Value.h"
#include "Generators/Perlin.h"
#include "Generators/Simplex.h"
#include "Generators/Cellular.h"
#include "Generators/Fractal.h"
#include "Generators/DomainWarp.h"
#include "Generators/DomainWarpSimplex.h"
#include "Generators/DomainWarpFractal.h"
#include "Generators/Modifiers.h"
#include "Generators/Blends.h"

namespace FastNoise
{
    namespace Internal
    {
        struct NodeAccess
        {
            template<typename T>
            static SmartNode<T> Make( T* object ) { return SmartNode<T>( object ); }
        };

        template<typename T, typename = void>
        struct IsConcrete : std::false_type {};

        template<typename T>
        struct IsConcrete<T, typename std::enable_if<std::is_same<typename T::FastNoiseConcreteType, T>::value>::type>
            : std::true_type {};

        template<typename T>
        Generator* AdoptAs( void* node ) { return new T( Adopt{}, node ); }

        // A node object of the node's own class around one reference to library node `node`.
        inline SmartNode<> AdoptNode( void* node )
        {
            using Factory = Generator* ( * )( void* );
            static const struct { const char* name; Factory make; } kClasses[] = {
                { "Constant", &AdoptAs<Constant> }, { "White", &AdoptAs<White> },
                { "Checkerboard", &AdoptAs<Checkerboard> }, { "SineWave", &AdoptAs<SineWave> },
                { "Gradient", &AdoptAs<Gradient> }, { "DistanceToPoint", &AdoptAs<DistanceToPoint> },
                { "Simplex", &AdoptAs<Simplex> }, { "SuperSimplex", &AdoptAs<SuperSimplex> },
                { "Perlin", &AdoptAs<Perlin> }, { "Value", &AdoptAs<Value> },
                { "CellularValue", &AdoptAs<CellularValue> }, { "CellularDistance", &AdoptAs<CellularDistance> },
                { "CellularLookup", &AdoptAs<CellularLookup> }, { "FractalFBm", &AdoptAs<FractalFBm> },
                { "PingPong", &AdoptAs<PingPong> }, { "FractalRidged", &AdoptAs<FractalRidged> },
                { "DomainWarpSimplex", &AdoptAs<DomainWarpSimplex> }, { "DomainWarpSuperSimplex", &AdoptAs<DomainWarpSuperSimplex> },
                { "DomainWarpGradient", &AdoptAs<DomainWarpGradient> },
                { "DomainWarpFractalProgressive", &AdoptAs<DomainWarpFractalProgressive> },
                { "DomainWarpFractalIndependent", &AdoptAs<DomainWarpFractalIndependent> },
                { "Add", &AdoptAs<Add> }, { "Subtract", &AdoptAs<Subtract> }, { "Multiply", &AdoptAs<Multiply> },
                { "Divide", &AdoptAs<Divide> }, { "Abs", &AdoptAs<Abs> }, { "Min", &AdoptAs<Min> }, { "Max", &AdoptAs<Max> },
                { "MinSmooth", &AdoptAs<MinSmooth> }, { "MaxSmooth", &AdoptAs<MaxSmooth> },
                { "SignedSquareRoot", &AdoptAs<SignedSquareRoot> }, { "PowFloat", &AdoptAs<PowFloat> },
                { "PowInt", &AdoptAs<PowInt> }, { "DomainScale", &AdoptAs<DomainScale> },
                { "DomainOffset", &AdoptAs<DomainOffset> }, { "DomainRotate", &AdoptAs<DomainRotate> },
                { "DomainAxisScale", &AdoptAs<DomainAxisScale> }, { "SeedOffset", &AdoptAs<SeedOffset> },
                { "ConvertRGBA8", &AdoptAs<ConvertRGBA8> }, { "GeneratorCache", &AdoptAs<GeneratorCache> },
                { "Fade", &AdoptAs<Fade> }, { "Remap", &AdoptAs<Remap> }, { "Terrace", &AdoptAs<Terrace> },
                { "AddDimension", &AdoptAs<AddDimension> }, { "RemoveDimension", &AdoptAs<RemoveDimension> },
                { "Modulus", &AdoptAs<Modulus> }, { "DomainRotatePlane", &AdoptAs<DomainRotatePlane> },
            };
            const char* name = fnGetMetadataName( fnGetMetadataID( node ) );
            for( const auto& c : kClasses )
            {
                if( std::strcmp( c.name, name ) == 0 )
                {
                    return NodeAccess::Make( c.make( node ) );
                }
            }
            fnDeleteNodeRef( node );
            return nullptr;
        }
    }

    // A new node of type T with the reference's defaults; null if the library could not create
    // it.  maxFeatureSet is accepted for source compatibility: the node always runs on the GPU.
    template<typename T>
    SmartNode<T> New( FastSIMD::FeatureSet /*maxFeatureSet*/ )
    {
        static_assert( std::is_base_of<Generator, T>::value, "This function should only be used for FastNoise node classes, for example FastNoise::Simplex" );
        static_assert( Internal::IsConcrete<T>::value, "Cannot create abstract node class, use a derived class, for example: Fractal -> FractalFBm" );

        T* object = new T();
        if( !object->GetNodeHandle() )
        {
            delete object;
            return nullptr;
        }
        return Internal::NodeAccess::Make( object );
    }

    // Root of the tree an encoded string describes (Node Editor "Copy Encoded Node Tree", or
    // Metadata::SerialiseNodeData), or null if the string is invalid.
    inline SmartNode<> NewFromEncodedNodeTree( const char* encodedNodeTreeString, FastSIMD::FeatureSet = FastSIMD::FeatureSet::Max )
    {
        void* node = encodedNodeTreeString ? fnNewFromEncodedNodeTree( encodedNodeTreeString, 0 ) : nullptr;
        return node ? Internal::AdoptNode( node ) : SmartNode<>( nullptr );
    }
}

#include "Metadata.h"
