// Fractal.h -- fractal nodes (reference include/FastNoise/Generators/Fractal.h: Fractal<T> :6-26,
// FractalFBm, FractalRidged).  Fractal<DomainWarp> is the base of the domain-warp fractals, whose
// source must be a domain warp node (the library refuses any other).
#pragma once
#include "Generator.h"

namespace FastNoise
{
    template<typename T = Generator>
    class Fractal : public virtual Generator
    {
    public:
        void SetSource( SmartNodeArg<T> gen )
        {
            this->SetNodeLookup( std::is_same<T, Generator>::value ? "Source" : "Domain Warp Source", gen );
        }
        void SetGain( float value ) { this->SetHybrid( "Gain", value ); }
        void SetGain( SmartNodeArg<> gen ) { this->SetHybrid( "Gain", gen ); }
        void SetWeightedStrength( float value ) { this->SetHybrid( "Weighted Strength", value ); }
        void SetWeightedStrength( SmartNodeArg<> gen ) { this->SetHybrid( "Weighted Strength", gen ); }
        void SetOctaveCount( int value ) { this->SetVariable( "Octaves", value ); }
        void SetLacunarity( float value ) { this->SetVariable( "Lacunarity", value ); }
    };

    class FractalFBm : public virtual Fractal<>
    {
        FASTNOISE_GB300_NODE( FractalFBm )
    };

    class FractalRidged : public virtual Fractal<>
    {
        FASTNOISE_GB300_NODE( FractalRidged )
    };
}
