// Config.h -- forward declarations of the C++ node API (reference include/FastNoise/Utility/Config.h).
//
// The reference takes FastSIMD::FeatureSet from its FastSIMD dependency: every node there is
// compiled once per CPU instruction set and New<T>() picks the best one.  Here every node is
// evaluated by CUDA kernels on the GPU, so a node has exactly one "feature set", the value
// fnGetActiveFeatureSet() reports (FN_GB300_FEATURE_SET).  The enum below keeps the names the
// reference's own headers use (Invalid, Max) so that calls such as New<T>() with the default
// argument, or an explicit FastSIMD::FeatureSet::Max, compile unchanged; the per-ISA names of
// FastSIMD are not provided, since this library has no CPU code path to select.
#pragma once
#include <cstdint>

#include "Export.h"

#define FASTNOISE_CALC_MIN_MAX true

namespace FastSIMD
{
    enum class FeatureSet : std::uint32_t
    {
        Invalid = 0,
        GB300 = 0x47423330u,        // FN_GB300_FEATURE_SET
        Max = 0xFFFFFFFFu,
    };
}

namespace FastNoise
{
    class Generator;
    struct Metadata;

    template<typename T = Generator>
    class SmartNode;

    // Setter argument type for node sources, as in the reference (Config.h:24-25).
    template<typename T = Generator>
    using SmartNodeArg = const SmartNode<const T>&;

    template<typename T>
    SmartNode<T> New( FastSIMD::FeatureSet maxFeatureSet = FastSIMD::FeatureSet::Max );
}

#include "SmartNode.h"
