// Blends.h -- operators and blends (reference include/FastNoise/Generators/Blends.h:
// OperatorSourceLHS :8-19, OperatorHybridLHS :33-45, Add, Subtract, Multiply, Divide, Modulus,
// Min, Max, PowFloat, PowInt, MinSmooth, MaxSmooth, Fade :291-324).
#pragma once
#include "Generator.h"

namespace FastNoise
{
    class OperatorSourceLHS : public virtual Generator
    {
    public:
        void SetLHS( SmartNodeArg<> gen ) { this->SetNodeLookup( "LHS", gen ); }
        void SetRHS( SmartNodeArg<> gen ) { this->SetHybrid( "RHS", gen ); }
        void SetRHS( float value ) { this->SetHybrid( "RHS", value ); }
    };

    class OperatorHybridLHS : public virtual Generator
    {
    public:
        void SetLHS( SmartNodeArg<> gen ) { this->SetHybrid( "LHS", gen ); }
        void SetLHS( float value ) { this->SetHybrid( "LHS", value ); }
        void SetRHS( SmartNodeArg<> gen ) { this->SetHybrid( "RHS", gen ); }
        void SetRHS( float value ) { this->SetHybrid( "RHS", value ); }
    };

    class Add : public virtual OperatorSourceLHS
    {
        FASTNOISE_GB300_NODE( Add )
    };

    class Subtract : public virtual OperatorHybridLHS
    {
        FASTNOISE_GB300_NODE( Subtract )
    };

    class Multiply : public virtual OperatorSourceLHS
    {
        FASTNOISE_GB300_NODE( Multiply )
    };

    class Divide : public virtual OperatorHybridLHS
    {
        FASTNOISE_GB300_NODE( Divide )
    };

    class Modulus : public virtual OperatorHybridLHS
    {
        FASTNOISE_GB300_NODE( Modulus )
    };

    class Min : public virtual OperatorSourceLHS
    {
        FASTNOISE_GB300_NODE( Min )
    };

    class Max : public virtual OperatorSourceLHS
    {
        FASTNOISE_GB300_NODE( Max )
    };

    class PowFloat : public virtual Generator
    {
        FASTNOISE_GB300_NODE( PowFloat )

        void SetValue( SmartNodeArg<> gen ) { this->SetHybrid( "Value", gen ); }
        void SetValue( float value ) { this->SetHybrid( "Value", value ); }
        void SetPow( SmartNodeArg<> gen ) { this->SetHybrid( "Pow", gen ); }
        void SetPow( float value ) { this->SetHybrid( "Pow", value ); }
    };

    class PowInt : public virtual Generator
    {
        FASTNOISE_GB300_NODE( PowInt )

        void SetValue( SmartNodeArg<> gen ) { this->SetNodeLookup( "Value", gen ); }
        void SetPow( int value ) { this->SetVariable( "Pow", value ); }
    };

    class MinSmooth : public virtual OperatorSourceLHS
    {
        FASTNOISE_GB300_NODE( MinSmooth )

        void SetSmoothness( SmartNodeArg<> gen ) { this->SetHybrid( "Smoothness", gen ); }
        void SetSmoothness( float value ) { this->SetHybrid( "Smoothness", value ); }
    };

    class MaxSmooth : public virtual OperatorSourceLHS
    {
        FASTNOISE_GB300_NODE( MaxSmooth )

        void SetSmoothness( SmartNodeArg<> gen ) { this->SetHybrid( "Smoothness", gen ); }
        void SetSmoothness( float value ) { this->SetHybrid( "Smoothness", value ); }
    };

    class Fade : public virtual Generator
    {
        FASTNOISE_GB300_NODE( Fade )

        enum class Interpolation
        {
            Linear,
            Hermite,
            Quintic,
        };

        void SetA( SmartNodeArg<> gen ) { this->SetNodeLookup( "A", gen ); }
        void SetB( SmartNodeArg<> gen ) { this->SetNodeLookup( "B", gen ); }

        void SetFade( SmartNodeArg<> gen ) { this->SetHybrid( "Fade", gen ); }
        void SetFade( float value ) { this->SetHybrid( "Fade", value ); }

        void SetFadeMin( SmartNodeArg<> gen ) { this->SetHybrid( "Fade Min", gen ); }
        void SetFadeMin( float value ) { this->SetHybrid( "Fade Min", value ); }

        void SetFadeMax( SmartNodeArg<> gen ) { this->SetHybrid( "Fade Max", gen ); }
        void SetFadeMax( float value ) { this->SetHybrid( "Fade Max", value ); }

        void SetInterpolation( Interpolation interpolation ) { this->SetVariable( "Interpolation", (int)interpolation ); }
    };
}
