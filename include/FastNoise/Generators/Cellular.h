// Cellular.h -- cellular (Voronoi) nodes (reference include/FastNoise/Generators/Cellular.h:
// Cellular<> :8-28, CellularValue :58-70, CellularDistance :88-113, CellularLookup :134-144).
#pragma once
#include "BasicGenerators.h"

namespace FastNoise
{
    template<typename PARENT = VariableRange<Seeded<ScalableGenerator>>>
    class Cellular : public virtual PARENT
    {
    public:
        void SetDistanceFunction( DistanceFunction value ) { this->SetVariable( "Distance Function", (int)value ); }

        void SetMinkowskiP( SmartNodeArg<> gen ) { this->SetHybrid( "Minkowski P", gen ); }
        void SetMinkowskiP( float value ) { this->SetHybrid( "Minkowski P", value ); }

        void SetGridJitter( SmartNodeArg<> gen ) { this->SetHybrid( "Grid Jitter", gen ); }
        void SetGridJitter( float value ) { this->SetHybrid( "Grid Jitter", value ); }

        void SetSizeJitter( SmartNodeArg<> gen ) { this->SetHybrid( "Size Jitter", gen ); }
        void SetSizeJitter( float value ) { this->SetHybrid( "Size Jitter", value ); }
    };

    class CellularValue : public virtual Cellular<>
    {
        FASTNOISE_GB300_NODE( CellularValue )

        static const int kMaxDistanceCount = 4;

        // clamped to [0, kMaxDistanceCount - 1] by the library, as by the reference
        void SetValueIndex( int value ) { this->SetVariable( "Value Index", value ); }
    };

    class CellularDistance : public virtual Cellular<>
    {
        FASTNOISE_GB300_NODE( CellularDistance )

        enum class ReturnType
        {
            Index0,
            Index0Add1,
            Index0Sub1,
            Index0Mul1,
            Index0Div1
        };

        static const int kMaxDistanceCount = 4;

        void SetDistanceIndex0( int value ) { this->SetVariable( "Distance Index 0", value ); }
        void SetDistanceIndex1( int value ) { this->SetVariable( "Distance Index 1", value ); }
        void SetReturnType( ReturnType value ) { this->SetVariable( "Return Type", (int)value ); }
    };

    class CellularLookup : public virtual Cellular<Seeded<ScalableGenerator>>
    {
        FASTNOISE_GB300_NODE( CellularLookup )

        void SetLookup( SmartNodeArg<> gen ) { this->SetNodeLookup( "Lookup", gen ); }
    };
}
