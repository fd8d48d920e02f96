// Perlin.h -- Perlin noise node (reference include/FastNoise/Generators/Perlin.h).
#pragma once
#include "BasicGenerators.h"

namespace FastNoise
{
    class Perlin : public virtual VariableRange<Seeded<ScalableGenerator>>
    {
        FASTNOISE_GB300_NODE( Perlin )
    };
}
