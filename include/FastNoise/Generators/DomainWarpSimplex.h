// DomainWarpSimplex.h -- simplex-based domain warps (reference
// include/FastNoise/Generators/DomainWarpSimplex.h:7-60).
#pragma once
#include "DomainWarp.h"

namespace FastNoise
{
    enum class VectorizationScheme
    {
        OrthogonalGradientMatrix,
        GradientOuterProduct
    };

    constexpr static const char* kVectorizationScheme_Strings[] =
        { "Orthogonal Gradient Matrix", "Gradient Outer Product" };

    class DomainWarpSimplex : public virtual DomainWarp
    {
        FASTNOISE_GB300_NODE( DomainWarpSimplex )

        void SetVectorizationScheme( VectorizationScheme value ) { this->SetVariable( "Vectorization Scheme", (int)value ); }
    };

    class DomainWarpSuperSimplex : public virtual DomainWarpSimplex
    {
        FASTNOISE_GB300_NODE( DomainWarpSuperSimplex )
    };
}
