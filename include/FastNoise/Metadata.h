// Metadata.h -- node metadata of the C++ API (reference include/FastNoise/Metadata.h: Metadata,
// its member descriptions, NodeData, SerialiseNodeData / DeserialiseNodeData).
//
// The table is read once from the library's metadata functions (fnGetMetadata*, FastNoise_C.h),
// which list the reference's node types, ids and members in the reference's order.  Member
// setters act on any node object of the matching type.  Encoded strings are produced and
// decoded by the library's codec (fnSerialiseNodeTree / fnNewFromEncodedNodeTree), whose byte
// format is the reference's (Metadata.cpp:88-308, Base64 with '@' runs).
#pragma once
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "Utility/Config.h"

namespace FastNoise
{
    struct NodeData;

    namespace Internal
    {
        struct MetadataTable;
        SmartNode<> AdoptNode( void* node );
    }

    struct Metadata
    {
        // Read-only sequence with the reference's iteration interface.
        template<typename T>
        class Vector
        {
        public:
            using const_iterator = const T*;

            const_iterator begin() const { return mItems.data(); }
            const_iterator end() const { return mItems.data() + mItems.size(); }
            size_t size() const { return mItems.size(); }
            const T& operator []( size_t i ) const { return mItems[i]; }

        private:
            friend struct Metadata;
            friend struct Internal::MetadataTable;
            std::vector<T> mItems;
        };

        struct NameDesc
        {
            const char* name;
            const char* desc;

            NameDesc( const char* name, const char* desc = "" ) : name( name ), desc( desc ) {}
        };

        struct Member
        {
            const char* name = "";
            const char* description = "";
            int dimensionIdx = -1;
        };

        struct MemberVariable : Member
        {
            enum eType
            {
                EFloat,
                EInt,
                EEnum
            };

            union ValueUnion
            {
                float f;
                int i;

                ValueUnion( float v = 0 ) { f = v; }
                ValueUnion( int v ) { i = v; }

                operator float() { return f; }
                operator int() { return i; }

                bool operator ==( const ValueUnion& rhs ) const { return i == rhs.i; }
            };

            eType type = EFloat;
            ValueUnion valueDefault, valueMin, valueMax;
            float valueUiDragSpeed = 0;
            Vector<const char*> enumNames;

            std::function<bool( Generator*, ValueUnion )> setFunc;
        };

        struct MemberNodeLookup : Member
        {
            std::function<bool( Generator*, SmartNodeArg<> )> setFunc;
        };

        struct MemberHybrid : Member
        {
            float valueDefault = 0;
            float valueUiDragSpeed = 0;

            std::function<bool( Generator*, float )> setValueFunc;
            std::function<bool( Generator*, SmartNodeArg<> )> setNodeFunc;
        };

        using node_id = uint8_t;

        virtual ~Metadata() = default;

        static const Vector<const Metadata*>& GetAll();

        static const Metadata* GetFromId( node_id nodeId )
        {
            const Vector<const Metadata*>& all = GetAll();
            return nodeId < all.size() ? all[nodeId] : nullptr;
        }

        template<typename T>
        static const Metadata& Get()
        {
            static_assert( std::is_base_of<Generator, T>::value, "Metadata::Get is for FastNoise node classes, for example FastNoise::Simplex" );
            return *GetFromId( (node_id)Internal::NodeId( T::MetadataName() ) );
        }

        // Encoded node tree of `nodeData` ("" when a node lookup is unset or the data does not
        // match its metadata).  fixUp: cut dependency loops and drop sources of the wrong type,
        // writing the changes back into the node data, as the reference's editor save does.
        static std::string SerialiseNodeData( NodeData* nodeData, bool fixUp = false );

        // Node data of an encoded tree (its nodes appended to nodeDataOut, which owns them);
        // nullptr when the string does not decode.  Shared nodes stay shared.
        static NodeData* DeserialiseNodeData( const char* serialisedBase64NodeData, std::vector<std::unique_ptr<NodeData>>& nodeDataOut );

        // "FractalFBm" -> "Fractal FBm"; removeGroups drops the node's group names ("FBm")
        static std::string FormatMetadataNodeName( const Metadata* metadata, bool removeGroups = false );

        // per-dimension members get their axis in front: "X Offset"
        static std::string FormatMetadataMemberName( const Member& member );

        virtual SmartNode<> CreateNode( FastSIMD::FeatureSet maxFeatureSet = FastSIMD::FeatureSet::Max ) const;

        node_id id = 0;
        Vector<MemberVariable> memberVariables;
        Vector<MemberNodeLookup> memberNodeLookups;
        Vector<MemberHybrid> memberHybrids;
        Vector<const char*> groups;

        const char* name = "";
        const char* description = "";
        const char* formattedName = nullptr;

    protected:
        static constexpr float kDefaultUiDragSpeedFloat = 0.02f;
        static constexpr float kDefaultUiDragSpeedInt = 0.2f;

        friend struct Internal::MetadataTable;
    };

    // Editable description of one node (the Node Editor's model): member values, sources and
    // hybrid inputs, each source another NodeData.
    struct NodeData
    {
        NodeData( const Metadata* data )
        {
            if( ( metadata = data ) )
            {
                for( const Metadata::MemberVariable& value : metadata->memberVariables )
                {
                    variables.push_back( value.valueDefault );
                }
                nodeLookups.assign( metadata->memberNodeLookups.size(), nullptr );
                for( const Metadata::MemberHybrid& value : metadata->memberHybrids )
                {
                    hybrids.emplace_back( nullptr, value.valueDefault );
                }
            }
        }

        const Metadata* metadata;
        std::vector<Metadata::MemberVariable::ValueUnion> variables;
        std::vector<NodeData*> nodeLookups;
        std::vector<std::pair<NodeData*, float>> hybrids;

        bool operator ==( const NodeData& rhs ) const
        {
            return metadata == rhs.metadata && variables == rhs.variables && nodeLookups == rhs.nodeLookups && hybrids == rhs.hybrids;
        }
    };
}

#include "Generators/Generator.h"

namespace FastNoise
{
    namespace Internal
    {
        inline int32_t FloatBits( float f ) { int32_t i; std::memcpy( &i, &f, 4 ); return i; }
        inline float BitsFloat( int32_t i ) { float f; std::memcpy( &f, &i, 4 ); return f; }

        // The metadata of every node type, built from the library's tables on first use.
        struct MetadataTable
        {
            struct Entry : Metadata
            {
            };

            std::vector<std::unique_ptr<Entry>> entries;
            Metadata::Vector<const Metadata*> all;

            MetadataTable()
            {
                int count = fnGetMetadataCount();
                for( int id = 0; id < count; id++ )
                {
                    std::unique_ptr<Entry> m( new Entry );
                    m->id = (Metadata::node_id)id;
                    m->name = fnGetMetadataName( id );
                    m->description = fnGetMetadataDescription( id );
                    for( int g = 0; g < fnGetMetadataGroupCount( id ); g++ )
                    {
                        m->groups.mItems.push_back( fnGetMetadataGroupName( id, g ) );
                    }
                    for( int i = 0; i < fnGetMetadataVariableCount( id ); i++ )
                    {
                        Metadata::MemberVariable v;
                        v.name = fnGetMetadataVariableName( id, i );
                        v.description = fnGetMetadataVariableDescription( id, i );
                        v.dimensionIdx = fnGetMetadataVariableDimensionIdx( id, i );
                        v.type = (Metadata::MemberVariable::eType)fnGetMetadataVariableType( id, i );
                        // the float getters hand back the raw bits of int members too
                        v.valueDefault.i = FloatBits( fnGetMetadataVariableDefaultFloat( id, i ) );
                        v.valueMin.i = FloatBits( fnGetMetadataVariableMinFloat( id, i ) );
                        v.valueMax.i = FloatBits( fnGetMetadataVariableMaxFloat( id, i ) );
                        v.valueUiDragSpeed = v.type == Metadata::MemberVariable::EFloat ? Metadata::kDefaultUiDragSpeedFloat
                                                                                       : Metadata::kDefaultUiDragSpeedInt;
                        for( int e = 0; e < fnGetMetadataEnumCount( id, i ); e++ )
                        {
                            v.enumNames.mItems.push_back( fnGetMetadataEnumName( id, i, e ) );
                        }
                        const bool isFloat = v.type == Metadata::MemberVariable::EFloat;
                        v.setFunc = [id, i, isFloat]( Generator* g, Metadata::MemberVariable::ValueUnion value )
                        {
                            if( !g || fnGetMetadataID( g->GetNodeHandle() ) != id )
                            {
                                return false;
                            }
                            return isFloat ? fnSetVariableFloat( g->GetNodeHandle(), i, value.f )
                                           : fnSetVariableIntEnum( g->GetNodeHandle(), i, value.i );
                        };
                        m->memberVariables.mItems.push_back( v );
                    }
                    for( int i = 0; i < fnGetMetadataNodeLookupCount( id ); i++ )
                    {
                        Metadata::MemberNodeLookup l;
                        l.name = fnGetMetadataNodeLookupName( id, i );
                        l.description = fnGetMetadataNodeLookupDescription( id, i );
                        l.dimensionIdx = fnGetMetadataNodeLookupDimensionIdx( id, i );
                        l.setFunc = [id, i]( Generator* g, SmartNodeArg<> gen )
                        {
                            return g && gen && fnGetMetadataID( g->GetNodeHandle() ) == id &&
                                   fnSetNodeLookup( g->GetNodeHandle(), i, gen->GetNodeHandle() );
                        };
                        m->memberNodeLookups.mItems.push_back( l );
                    }
                    for( int i = 0; i < fnGetMetadataHybridCount( id ); i++ )
                    {
                        Metadata::MemberHybrid h;
                        h.name = fnGetMetadataHybridName( id, i );
                        h.description = fnGetMetadataHybridDescription( id, i );
                        h.dimensionIdx = fnGetMetadataHybridDimensionIdx( id, i );
                        h.valueDefault = fnGetMetadataHybridDefault( id, i );
                        h.valueUiDragSpeed = Metadata::kDefaultUiDragSpeedFloat;
                        h.setValueFunc = [id, i]( Generator* g, float value )
                        {
                            return g && fnGetMetadataID( g->GetNodeHandle() ) == id && fnSetHybridFloat( g->GetNodeHandle(), i, value );
                        };
                        h.setNodeFunc = [id, i]( Generator* g, SmartNodeArg<> gen )
                        {
                            return g && gen && fnGetMetadataID( g->GetNodeHandle() ) == id &&
                                   fnSetHybridNodeLookup( g->GetNodeHandle(), i, gen->GetNodeHandle() );
                        };
                        m->memberHybrids.mItems.push_back( h );
                    }
                    all.mItems.push_back( m.get() );
                    entries.push_back( std::move( m ) );
                }
            }

            static const MetadataTable& Get()
            {
                static const MetadataTable table;
                return table;
            }
        };

        // Library nodes made from node data for one serialisation; released on destruction.
        struct NodeDataBuilder
        {
            bool fixUp;
            std::unordered_map<const NodeData*, void*> made;

            ~NodeDataBuilder()
            {
                for( auto& kv : made )
                {
                    fnDeleteNodeRef( kv.second );
                }
            }

            // `path`: the nodes between the root and this one (a source found on it is a loop)
            void* Build( NodeData* nodeData, std::unordered_set<const NodeData*> path )
            {
                const Metadata* metadata = nodeData ? nodeData->metadata : nullptr;
                if( !metadata || nodeData->variables.size() != metadata->memberVariables.size() ||
                    nodeData->nodeLookups.size() != metadata->memberNodeLookups.size() ||
                    nodeData->hybrids.size() != metadata->memberHybrids.size() )
                {
                    return nullptr;
                }
                path.insert( nodeData );
                if( fixUp )
                {
                    for( auto& lookup : nodeData->nodeLookups )
                    {
                        if( path.count( lookup ) ) lookup = nullptr;
                    }
                    for( auto& hybrid : nodeData->hybrids )
                    {
                        if( path.count( hybrid.first ) ) hybrid.first = nullptr;
                    }
                }
                auto found = made.find( nodeData );
                if( found != made.end() )
                {
                    return found->second;                       // a shared node: encoded once, then referenced
                }
                void* node = fnNewFromMetadata( metadata->id, 0 );
                if( !node )
                {
                    return nullptr;
                }
                made[nodeData] = node;
                for( size_t i = 0; i < metadata->memberVariables.size(); i++ )
                {
                    const bool isFloat = metadata->memberVariables[i].type == Metadata::MemberVariable::EFloat;
                    bool ok = isFloat ? fnSetVariableFloat( node, (int)i, BitsFloat( nodeData->variables[i].i ) )
                                      : fnSetVariableIntEnum( node, (int)i, nodeData->variables[i].i );
                    if( !ok ) return nullptr;
                }
                for( size_t i = 0; i < metadata->memberNodeLookups.size(); i++ )
                {
                    NodeData* source = nodeData->nodeLookups[i];
                    if( !source || path.count( source ) ) return nullptr;     // unset, or a loop left without fixUp
                    void* child = Build( source, path );
                    if( !child ) return nullptr;
                    if( !fnSetNodeLookup( node, (int)i, child ) )
                    {
                        if( fixUp ) nodeData->nodeLookups[i] = nullptr;      // a source of the wrong type
                        return nullptr;
                    }
                }
                for( size_t i = 0; i < metadata->memberHybrids.size(); i++ )
                {
                    NodeData* source = nodeData->hybrids[i].first;
                    if( !source )
                    {
                        if( !fnSetHybridFloat( node, (int)i, nodeData->hybrids[i].second ) ) return nullptr;
                        continue;
                    }
                    if( path.count( source ) ) return nullptr;
                    void* child = Build( source, path );
                    if( !child ) return nullptr;
                    if( !fnSetHybridNodeLookup( node, (int)i, child ) )
                    {
                        if( fixUp ) nodeData->hybrids[i].first = nullptr;
                        return nullptr;
                    }
                }
                return node;
            }
        };

        // Node data of library node `node` (and its sources), sharing repeated nodes.
        inline NodeData* ReadNodeData( void* node, std::unordered_map<void*, NodeData*>& seen,
                                       std::vector<std::unique_ptr<NodeData>>& out )
        {
            auto found = seen.find( node );
            if( found != seen.end() ) return found->second;
            const Metadata* metadata = Metadata::GetFromId( (Metadata::node_id)fnGetMetadataID( node ) );
            if( !metadata ) return nullptr;
            out.emplace_back( new NodeData( metadata ) );
            NodeData* data = out.back().get();
            seen[node] = data;
            for( size_t i = 0; i < data->variables.size(); i++ )
            {
                int bits = 0;
                if( fnGetVariableBits( node, (int)i, &bits ) == FN_OK ) data->variables[i].i = bits;
            }
            for( size_t i = 0; i < data->nodeLookups.size(); i++ )
            {
                void* child = fnGetNodeLookupRef( node, (int)i );
                if( child )
                {
                    data->nodeLookups[i] = ReadNodeData( child, seen, out );
                    fnDeleteNodeRef( child );                       // the tree keeps its own reference
                }
            }
            for( size_t i = 0; i < data->hybrids.size(); i++ )
            {
                float value = data->hybrids[i].second;
                fnGetHybridFloat( node, (int)i, &value );
                data->hybrids[i].second = value;
                void* child = fnGetHybridNodeLookupRef( node, (int)i );
                if( child )
                {
                    data->hybrids[i].first = ReadNodeData( child, seen, out );
                    fnDeleteNodeRef( child );
                }
            }
            return data;
        }
    }

    inline const Metadata::Vector<const Metadata*>& Metadata::GetAll()
    {
        return Internal::MetadataTable::Get().all;
    }

    inline SmartNode<> Metadata::CreateNode( FastSIMD::FeatureSet ) const
    {
        void* node = fnNewFromMetadata( id, 0 );
        return node ? Internal::AdoptNode( node ) : SmartNode<>( nullptr );
    }

    inline std::string Metadata::SerialiseNodeData( NodeData* nodeData, bool fixUp )
    {
        Internal::NodeDataBuilder builder{ fixUp, {} };
        void* root = builder.Build( nodeData, {} );
        if( !root ) return "";
        int length = fnSerialiseNodeTree( root, nullptr, 0 );
        if( length < 0 ) return "";
        std::string encoded( (size_t)length + 1, '\0' );
        if( fnSerialiseNodeTree( root, &encoded[0], length + 1 ) != length ) return "";
        encoded.resize( (size_t)length );
        return encoded;
    }

    inline NodeData* Metadata::DeserialiseNodeData( const char* serialisedBase64NodeData, std::vector<std::unique_ptr<NodeData>>& nodeDataOut )
    {
        void* root = serialisedBase64NodeData ? fnNewFromEncodedNodeTree( serialisedBase64NodeData, 0 ) : nullptr;
        if( !root ) return nullptr;
        std::unordered_map<void*, NodeData*> seen;
        NodeData* data = Internal::ReadNodeData( root, seen, nodeDataOut );
        fnDeleteNodeRef( root );
        return data;
    }

    inline std::string Metadata::FormatMetadataNodeName( const Metadata* metadata, bool removeGroups )
    {
        std::string text = metadata->formattedName ? metadata->formattedName : "";
        if( !metadata->formattedName )
        {
            // a space where a lower-case letter meets a capital or a digit
            const std::string raw = metadata->name;
            for( size_t i = 0; i < raw.size(); i++ )
            {
                const char c = raw[i];
                const bool starts = i > 0 && ( ( c >= 'A' && c <= 'Z' ) || ( c >= '0' && c <= '9' ) ) &&
                                    raw[i - 1] >= 'a' && raw[i - 1] <= 'z';
                if( starts ) text += ' ';
                text += c;
            }
        }
        if( removeGroups )
        {
            for( const char* group : metadata->groups )
            {
                size_t at = text.find( group );
                if( at != std::string::npos ) text.erase( at, std::strlen( group ) + 1 );
            }
        }
        return text.empty() ? std::string( metadata->name ) : text;
    }

    inline std::string Metadata::FormatMetadataMemberName( const Member& member )
    {
        if( member.dimensionIdx < 0 || member.dimensionIdx >= (int)Dim::Count ) return member.name;
        return std::string( kDim_Strings[member.dimensionIdx] ) + " " + member.name;
    }

    inline const Metadata& Generator::GetMetadata() const
    {
        return *Metadata::GetFromId( (Metadata::node_id)fnGetMetadataID( mNode ) );
    }
}

#include "FastNoise.h"
