// BasicGenerators.h -- member mixins and basic nodes (reference include/FastNoise/Generators/
// BasicGenerators.h: ScalableGenerator :14-30, Seeded :51-66, VariableRange :89-114, Constant,
// White, Checkerboard, SineWave, Gradient, DistanceToPoint).  Setters forward to the node's
// metadata members, whose side effects (frequency = 1 / scale, the output-range scale) the
// library applies exactly as the reference's setters do.
#pragma once
#include "Generator.h"

namespace FastNoise
{
    class ScalableGenerator : public virtual Generator
    {
    public:
        void SetScale( float value ) { this->SetVariable( "Feature Scale", value ); }
    };

    template<typename PARENT>
    class Seeded : public virtual PARENT
    {
    public:
        void SetSeedOffset( int value ) { this->SetVariable( "Seed Offset", value ); }
    };

    template<typename PARENT>
    class VariableRange : public virtual PARENT
    {
    public:
        void SetOutputMin( float value ) { this->SetVariable( "Output Min", value ); }
        void SetOutputMax( float value ) { this->SetVariable( "Output Max", value ); }
    };

    class Constant : public virtual Generator
    {
        FASTNOISE_GB300_NODE( Constant )

        void SetValue( float value ) { this->SetVariable( "Value", value ); }
    };

    class White : public virtual VariableRange<Seeded<Generator>>
    {
        FASTNOISE_GB300_NODE( White )
    };

    class Checkerboard : public virtual VariableRange<ScalableGenerator>
    {
        FASTNOISE_GB300_NODE( Checkerboard )
    };

    class SineWave : public virtual VariableRange<ScalableGenerator>
    {
        FASTNOISE_GB300_NODE( SineWave )
    };

    class Gradient : public virtual Generator
    {
        FASTNOISE_GB300_NODE( Gradient )

        template<Dim D>
        void SetMultiplier( float multiplier ) { this->SetVariable( "Multiplier", multiplier, (int)D ); }
        template<Dim D>
        void SetOffset( float offset ) { this->SetHybrid( "Offset", offset, (int)D ); }
        template<Dim D>
        void SetOffset( SmartNodeArg<> gen ) { this->SetHybrid( "Offset", gen, (int)D ); }
    };

    class DistanceToPoint : public virtual Generator
    {
        FASTNOISE_GB300_NODE( DistanceToPoint )

        // The reference keeps this source without evaluating it (its metadata has no Source
        // member); the node object holds it the same way.
        void SetSource( SmartNodeArg<> gen ) { mSource = gen; }
        void SetDistanceFunction( DistanceFunction value ) { this->SetVariable( "Distance Function", (int)value ); }

        void SetMinkowskiP( SmartNodeArg<> gen ) { this->SetHybrid( "Minkowski P", gen ); }
        void SetMinkowskiP( float value ) { this->SetHybrid( "Minkowski P", value ); }

        void SetPoint( float x, float y, float z = 0, float w = 0 )
        {
            this->SetHybrid( "Point", x, 0 );
            this->SetHybrid( "Point", y, 1 );
            this->SetHybrid( "Point", z, 2 );
            this->SetHybrid( "Point", w, 3 );
        }

        template<Dim D>
        void SetPoint( float value ) { this->SetHybrid( "Point", value, (int)D ); }

        template<Dim D>
        void SetPoint( SmartNodeArg<> gen ) { this->SetHybrid( "Point", gen, (int)D ); }

    private:
        SmartNode<const Generator> mSource;
    };
}
