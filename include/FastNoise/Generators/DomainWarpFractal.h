// DomainWarpFractal.h -- fractal domain warps (reference
// include/FastNoise/Generators/DomainWarpFractal.h: Progressive :7-30, Independent :33-56).
#pragma once
#include "Fractal.h"
#include "DomainWarp.h"

namespace FastNoise
{
    class DomainWarpFractalProgressive : public virtual Fractal<DomainWarp>
    {
        FASTNOISE_GB300_NODE( DomainWarpFractalProgressive )
    };

    class DomainWarpFractalIndependent : public virtual Fractal<DomainWarp>
    {
        FASTNOISE_GB300_NODE( DomainWarpFractalIndependent )
    };
}
