// Simplex.h -- Simplex and SuperSimplex (OpenSimplex2S) noise nodes (reference
// include/FastNoise/Generators/Simplex.h).
#pragma once
#include "BasicGenerators.h"

namespace FastNoise
{
    class Simplex : public virtual VariableRange<Seeded<ScalableGenerator>>
    {
        FASTNOISE_GB300_NODE( Simplex )
    };

    class SuperSimplex : public virtual VariableRange<Seeded<ScalableGenerator>>
    {
        FASTNOISE_GB300_NODE( SuperSimplex )
    };
}
