// Modifiers.h -- domain modifiers and output modifiers (reference
// include/FastNoise/Generators/Modifiers.h: DomainScale, DomainOffset, DomainRotate, SeedOffset,
// Remap, ConvertRGBA8, Terrace, PingPong, DomainAxisScale, AddDimension, RemoveDimension,
// GeneratorCache, SignedSquareRoot, Abs, DomainRotatePlane).
#pragma once
#include "Generator.h"

namespace FastNoise
{
    class DomainScale : public virtual Generator
    {
        FASTNOISE_GB300_NODE( DomainScale )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetScaling( float value ) { this->SetVariable( "Scaling", value ); }
    };

    class DomainOffset : public virtual Generator
    {
        FASTNOISE_GB300_NODE( DomainOffset )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }

        template<Dim D>
        void SetOffset( float value ) { this->SetHybrid( "Offset", value, (int)D ); }

        template<Dim D>
        void SetOffset( SmartNodeArg<> gen ) { this->SetHybrid( "Offset", gen, (int)D ); }
    };

    class DomainRotate : public virtual Generator
    {
        FASTNOISE_GB300_NODE( DomainRotate )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }

        // radians; the rotation matrix is rebuilt by the library as by the reference's setters
        void SetYaw( float value ) { this->SetVariable( "Yaw", value ); }
        void SetPitch( float value ) { this->SetVariable( "Pitch", value ); }
        void SetRoll( float value ) { this->SetVariable( "Roll", value ); }
    };

    class SeedOffset : public virtual Generator
    {
        FASTNOISE_GB300_NODE( SeedOffset )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetOffset( int value ) { this->SetVariable( "Seed Offset", value ); }
    };

    class Remap : public virtual Generator
    {
        FASTNOISE_GB300_NODE( Remap )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }

        void SetFromMin( float value ) { this->SetHybrid( "From Min", value ); }
        void SetFromMin( SmartNodeArg<> gen ) { this->SetHybrid( "From Min", gen ); }

        void SetFromMax( float value ) { this->SetHybrid( "From Max", value ); }
        void SetFromMax( SmartNodeArg<> gen ) { this->SetHybrid( "From Max", gen ); }

        void SetToMin( float value ) { this->SetHybrid( "To Min", value ); }
        void SetToMin( SmartNodeArg<> gen ) { this->SetHybrid( "To Min", gen ); }

        void SetToMax( float value ) { this->SetHybrid( "To Max", value ); }
        void SetToMax( SmartNodeArg<> gen ) { this->SetHybrid( "To Max", gen ); }

        void SetClampOutput( Boolean value ) { this->SetVariable( "Clamp Output", (int)value ); }
        void SetClampOutput( bool value ) { SetClampOutput( value ? Boolean::True : Boolean::False ); }
    };

    class ConvertRGBA8 : public virtual Generator
    {
        FASTNOISE_GB300_NODE( ConvertRGBA8 )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetMinMax( float min, float max )
        {
            this->SetVariable( "Min", min );
            this->SetVariable( "Max", max );
        }
    };

    class Terrace : public virtual Generator
    {
        FASTNOISE_GB300_NODE( Terrace )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetStepCount( float stepCount ) { this->SetVariable( "Step Count", stepCount ); }

        void SetSmoothness( float smoothness ) { this->SetHybrid( "Smoothness", smoothness ); }
        void SetSmoothness( SmartNodeArg<> gen ) { this->SetHybrid( "Smoothness", gen ); }
    };

    class PingPong : public virtual Generator
    {
        FASTNOISE_GB300_NODE( PingPong )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }

        void SetPingPongStrength( float value ) { this->SetHybrid( "Ping Pong Strength", value ); }
        void SetPingPongStrength( SmartNodeArg<> gen ) { this->SetHybrid( "Ping Pong Strength", gen ); }
    };

    class DomainAxisScale : public virtual Generator
    {
        FASTNOISE_GB300_NODE( DomainAxisScale )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }

        template<Dim D>
        void SetScaling( float value ) { this->SetVariable( "Scaling", value, (int)D ); }
    };

    class AddDimension : public virtual Generator
    {
        FASTNOISE_GB300_NODE( AddDimension )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetNewDimensionPosition( float value ) { this->SetHybrid( "New Dimension Position", value ); }
        void SetNewDimensionPosition( SmartNodeArg<> gen ) { this->SetHybrid( "New Dimension Position", gen ); }
    };

    class RemoveDimension : public virtual Generator
    {
        FASTNOISE_GB300_NODE( RemoveDimension )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetRemoveDimension( Dim dimension ) { this->SetVariable( "Remove Dimension", (int)dimension ); }
    };

    class GeneratorCache : public virtual Generator
    {
        FASTNOISE_GB300_NODE( GeneratorCache )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
    };

    class SignedSquareRoot : public virtual Generator
    {
        FASTNOISE_GB300_NODE( SignedSquareRoot )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
    };

    class Abs : public virtual Generator
    {
        FASTNOISE_GB300_NODE( Abs )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
    };

    enum class PlaneRotationType
    {
        ImproveXYPlanes,
        ImproveXZPlanes
    };

    constexpr static const char* kPlaneRotationType_Strings[] = { "Improve XY Planes", "Improve XZ Planes" };

    class DomainRotatePlane : public virtual Generator
    {
        FASTNOISE_GB300_NODE( DomainRotatePlane )

        void SetSource( SmartNodeArg<> gen ) { this->SetNodeLookup( "Source", gen ); }
        void SetRotationType( PlaneRotationType type ) { this->SetVariable( "Rotation Type", (int)type ); }
    };
}
