// Value.h -- Value noise node (reference include/FastNoise/Generators/Value.h).
#pragma once
#include "BasicGenerators.h"

namespace FastNoise
{
    class Value : public virtual VariableRange<Seeded<ScalableGenerator>>
    {
        FASTNOISE_GB300_NODE( Value )
    };
}
