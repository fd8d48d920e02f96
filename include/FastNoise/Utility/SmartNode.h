// SmartNode.h -- reference-counted node handle of the C++ API (reference
// include/FastNoise/Utility/SmartNode.h:71-320: same class name, constructors, conversions,
// DynamicCast, get/reset/swap/use_count).
//
// A node object here is a small C++ wrapper that owns one reference to a node of
// libfastnoise_gb300.so (the C-ABI handle).  SmartNode counts references to the wrapper with an
// atomic counter kept in the wrapper; the last SmartNode deletes the wrapper, which drops its
// library reference.  Sources set on a node are held by the library tree itself, so a child's
// wrapper may go away while the parent still uses the child.
#pragma once
#include <cassert>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <type_traits>
#include <utility>

#include "Config.h"

namespace FastNoise
{
    class SmartNodeManager
    {
    public:
        static constexpr uint64_t kInvalidReferenceId = (uint64_t)0;

        SmartNodeManager() = delete;

        // The reference allocates node objects from a pool it lets callers size.  Node objects
        // here are plain heap objects (the node state lives in the GPU library), so there is
        // no pool and the call has no effect.
        static void SetMemoryPoolSize( uint32_t ) {}
    };

    namespace Internal
    {
        struct NodeAccess;
    }

    template<typename T>
    class SmartNode
    {
    public:
        static_assert( std::is_base_of<Generator, T>::value, "SmartNode should only be used for FastNoise node classes" );

        // nullptr when `node` is not a T (dynamic_cast on the node object)
        template<typename U>
        static SmartNode DynamicCast( const SmartNode<U>& node )
        {
            return SmartNode( dynamic_cast<T*>( node.mPtr ) );
        }

        constexpr SmartNode( std::nullptr_t = nullptr ) noexcept : mPtr( nullptr ) {}

        SmartNode( const SmartNode& node ) noexcept : mPtr( node.mPtr ) { Acquire( mPtr ); }

        template<typename U, typename = typename std::enable_if<std::is_convertible<U*, T*>::value>::type>
        SmartNode( const SmartNode<U>& node ) noexcept : mPtr( node.mPtr ) { Acquire( mPtr ); }

        // shares the reference count of `owner` while pointing at `ptr` (an object inside it)
        template<typename U>
        SmartNode( const SmartNode<U>&, T* ptr ) noexcept : mPtr( ptr ) { Acquire( mPtr ); }

        SmartNode( SmartNode&& node ) noexcept : mPtr( node.mPtr ) { node.mPtr = nullptr; }

        template<typename U, typename = typename std::enable_if<std::is_convertible<U*, T*>::value>::type>
        SmartNode( SmartNode<U>&& node ) noexcept : mPtr( node.mPtr ) { node.mPtr = nullptr; }

        ~SmartNode() { Release(); }

        SmartNode& operator=( SmartNode&& node ) noexcept
        {
            swap( node );
            return *this;
        }

        template<typename U, typename = typename std::enable_if<std::is_convertible<U*, T*>::value>::type>
        SmartNode& operator=( SmartNode<U>&& node ) noexcept
        {
            if( mPtr != node.mPtr )
            {
                Release();
                mPtr = node.mPtr;
                node.mPtr = nullptr;
            }
            return *this;
        }

        SmartNode& operator=( const SmartNode& node ) noexcept
        {
            if( mPtr != node.mPtr )
            {
                Acquire( node.mPtr );
                Release();
                mPtr = node.mPtr;
            }
            return *this;
        }

        template<typename U, typename = typename std::enable_if<std::is_convertible<U*, T*>::value>::type>
        SmartNode& operator=( const SmartNode<U>& node ) noexcept
        {
            if( mPtr != node.mPtr )
            {
                Acquire( node.mPtr );
                Release();
                mPtr = node.mPtr;
            }
            return *this;
        }

        template<typename U>
        friend bool operator==( const SmartNode& lhs, const SmartNode<U>& rhs ) noexcept { return lhs.get() == rhs.get(); }

        template<typename U>
        friend bool operator!=( const SmartNode& lhs, const SmartNode<U>& rhs ) noexcept { return lhs.get() != rhs.get(); }

        const T& operator*() const noexcept { assert( mPtr ); return *mPtr; }
        T& operator*() noexcept { assert( mPtr ); return *mPtr; }
        const T* operator->() const noexcept { assert( mPtr ); return mPtr; }
        T* operator->() noexcept { assert( mPtr ); return mPtr; }

        explicit operator bool() const noexcept { return mPtr != nullptr; }

        const T* get() const noexcept { return mPtr; }
        T* get() noexcept { return mPtr; }

        void reset( T* ptr = nullptr )
        {
            *this = SmartNode( ptr );
        }

        void swap( SmartNode& node ) noexcept { std::swap( mPtr, node.mPtr ); }

        long use_count() const noexcept { return mPtr ? (long)mPtr->RefAdd( 0 ) : 0; }

        bool unique() const noexcept { return use_count() == 1; }

    private:
        template<typename U>
        friend class SmartNode;
        friend struct Internal::NodeAccess;

        explicit SmartNode( T* ptr ) noexcept : mPtr( ptr ) { Acquire( ptr ); }

        static void Acquire( T* ptr ) noexcept
        {
            if( ptr )
            {
                ptr->RefAdd( 1 );
            }
        }

        void Release() noexcept
        {
            if( mPtr )
            {
                if( mPtr->RefAdd( -1 ) == 1 )
                {
                    delete mPtr;
                }
                mPtr = nullptr;
            }
        }

        T* mPtr;
    };
}

namespace std
{
    template<typename T>
    struct hash<FastNoise::SmartNode<T>>
    {
        size_t operator()( const FastNoise::SmartNode<T>& node ) const noexcept
        {
            return std::hash<const T*>()( node.get() );
        }
    };
}
