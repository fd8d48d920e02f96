// DomainWarp.h -- domain warp base and DomainWarpGradient (reference
// include/FastNoise/Generators/DomainWarp.h:6-45).
#pragma once
#include "BasicGenerators.h"

namespace FastNoise
{
    class DomainWarp : public virtual Seeded<ScalableGenerator>
    {
    public:
        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetWarpAmplitude( SmartNodeArg<> gen ) { this->SetHybrid( "Warp Amplitude", gen ); }
        void SetWarpAmplitude( float value ) { this->SetHybrid( "Warp Amplitude", value ); }

        template<Dim D>
        void SetAmplitudeScaling( float value ) { this->SetVariable( "Amplitude Scaling", value, (int)D ); }
    };

    class DomainWarpGradient : public virtual DomainWarp
    {
        FASTNOISE_GB300_NODE( DomainWarpGradient )
    };
}
