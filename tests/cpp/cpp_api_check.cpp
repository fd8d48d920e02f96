// cpp_api_check.cpp -- test driver for the C++ node API (include/FastNoise/FastNoise.h).
//
// Built and run by tests/test_cpp_api.py (CPU checks) and tests/test_gpu_cpp_api.py (GPU).
//   cpp_api_check meta                 metadata, New<T> for every node class, DynamicCast,
//                                      setter effects seen through the encoded tree,
//                                      NodeData round trips (no GPU needed)
//   cpp_api_check encode               prints the encoded trees of the workload trees built
//                                      with New<T> and setters, one per line
//   cpp_api_check gen DIR              generates the workload trees through the C++ API, built
//                                      both with setters and from their encoded strings, and
//                                      writes DIR/<name>.f32 (values) and DIR/<name>.mm (min, max)
//   cpp_api_check threads N            N host threads generate on one shared tree at once while
//                                      the library specialises it in the background; every
//                                      result must equal the single-thread result bit for bit
#include <FastNoise/FastNoise.h>
#include <FastNoise/Metadata.h>

#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <thread>
#include <vector>

using namespace FastNoise;

static int g_failures = 0;

#define CHECK( cond )                                                                 \
    do                                                                                \
    {                                                                                 \
        if( !( cond ) )                                                               \
        {                                                                             \
            std::fprintf( stderr, "CHECK failed at line %d: %s\n", __LINE__, #cond ); \
            ++g_failures;                                                             \
        }                                                                             \
    } while( 0 )

static std::string Encode( const Generator* g )
{
    int n = fnSerialiseNodeTree( g->GetNodeHandle(), nullptr, 0 );
    if( n < 0 ) return "";
    std::string s( (size_t)n + 1, '\0' );
    fnSerialiseNodeTree( g->GetNodeHandle(), &s[0], n + 1 );
    s.resize( (size_t)n );
    return s;
}

// ---- the workload trees, built with the reference's setters ----

static SmartNode<> SimplexC0()
{
    auto simplex = New<Simplex>();
    simplex->SetScale( 50.0f );                            // frequency 0.02
    return simplex;
}

static SmartNode<> FbmPerlinC1()
{
    auto fbm = New<FractalFBm>();
    fbm->SetSource( New<Perlin>() );
    fbm->SetOctaveCount( 5 );
    fbm->SetGain( 0.5f );
    fbm->SetLacunarity( 2.0f );
    fbm->SetWeightedStrength( 0.0f );
    return fbm;
}

static SmartNode<> TerrainC2()
{
    auto ridged = New<FractalRidged>();
    ridged->SetSource( New<SuperSimplex>() );
    ridged->SetOctaveCount( 4 );
    auto warp = New<DomainWarpGradient>();
    warp->SetSource( ridged );
    warp->SetWarpAmplitude( 30.0f );
    auto warpFractal = New<DomainWarpFractalProgressive>();
    warpFractal->SetSource( warp );
    warpFractal->SetOctaveCount( 3 );
    auto cells = New<CellularDistance>();
    cells->SetDistanceFunction( DistanceFunction::Euclidean );
    cells->SetDistanceIndex0( 0 );
    cells->SetDistanceIndex1( 1 );
    cells->SetReturnType( CellularDistance::ReturnType::Index0Sub1 );
    cells->SetGridJitter( 1.0f );
    auto fade = New<Fade>();
    fade->SetA( warpFractal );
    fade->SetB( cells );
    auto remap = New<Remap>();
    remap->SetSource( fade );
    remap->SetFromMin( -1.0f );
    remap->SetFromMax( 1.0f );
    remap->SetToMin( 0.0f );
    remap->SetToMax( 1.0f );
    auto terrace = New<Terrace>();
    terrace->SetSource( remap );
    terrace->SetStepCount( 8.0f );
    terrace->SetSmoothness( 0.3f );
    return terrace;
}

static SmartNode<> BlendTree()
{
    auto mul = New<Multiply>();
    mul->SetLHS( New<Perlin>() );
    mul->SetRHS( New<Value>() );
    auto add = New<Add>();
    add->SetLHS( New<Simplex>() );
    add->SetRHS( mul );
    return add;
}

// ---- meta ----

template<typename T>
static void CheckClass( const char* name )
{
    SmartNode<T> node = New<T>();
    CHECK( node );
    if( !node ) return;
    CHECK( std::strcmp( node->GetMetadata().name, name ) == 0 );
    CHECK( &Metadata::Get<T>() == &node->GetMetadata() );
    CHECK( node->GetActiveFeatureSet() == FastSIMD::FeatureSet::GB300 );
    SmartNode<> base = node;
    CHECK( base.use_count() == 2 );
    CHECK( SmartNode<T>::DynamicCast( base ) == node );
    SmartNode<> made = node->GetMetadata().CreateNode();
    CHECK( made && std::strcmp( made->GetMetadata().name, name ) == 0 );
    CHECK( SmartNode<T>::DynamicCast( made ) );
}

static int Meta()
{
    CheckClass<Constant>( "Constant" );
    CheckClass<White>( "White" );
    CheckClass<Checkerboard>( "Checkerboard" );
    CheckClass<SineWave>( "SineWave" );
    CheckClass<Gradient>( "Gradient" );
    CheckClass<DistanceToPoint>( "DistanceToPoint" );
    CheckClass<Simplex>( "Simplex" );
    CheckClass<SuperSimplex>( "SuperSimplex" );
    CheckClass<Perlin>( "Perlin" );
    CheckClass<Value>( "Value" );
    CheckClass<CellularValue>( "CellularValue" );
    CheckClass<CellularDistance>( "CellularDistance" );
    CheckClass<CellularLookup>( "CellularLookup" );
    CheckClass<FractalFBm>( "FractalFBm" );
    CheckClass<PingPong>( "PingPong" );
    CheckClass<FractalRidged>( "FractalRidged" );
    CheckClass<DomainWarpSimplex>( "DomainWarpSimplex" );
    CheckClass<DomainWarpSuperSimplex>( "DomainWarpSuperSimplex" );
    CheckClass<DomainWarpGradient>( "DomainWarpGradient" );
    CheckClass<DomainWarpFractalProgressive>( "DomainWarpFractalProgressive" );
    CheckClass<DomainWarpFractalIndependent>( "DomainWarpFractalIndependent" );
    CheckClass<Add>( "Add" );
    CheckClass<Subtract>( "Subtract" );
    CheckClass<Multiply>( "Multiply" );
    CheckClass<Divide>( "Divide" );
    CheckClass<Abs>( "Abs" );
    CheckClass<Min>( "Min" );
    CheckClass<Max>( "Max" );
    CheckClass<MinSmooth>( "MinSmooth" );
    CheckClass<MaxSmooth>( "MaxSmooth" );
    CheckClass<SignedSquareRoot>( "SignedSquareRoot" );
    CheckClass<PowFloat>( "PowFloat" );
    CheckClass<PowInt>( "PowInt" );
    CheckClass<DomainScale>( "DomainScale" );
    CheckClass<DomainOffset>( "DomainOffset" );
    CheckClass<DomainRotate>( "DomainRotate" );
    CheckClass<DomainAxisScale>( "DomainAxisScale" );
    CheckClass<SeedOffset>( "SeedOffset" );
    CheckClass<ConvertRGBA8>( "ConvertRGBA8" );
    CheckClass<GeneratorCache>( "GeneratorCache" );
    CheckClass<Fade>( "Fade" );
    CheckClass<Remap>( "Remap" );
    CheckClass<Terrace>( "Terrace" );
    CheckClass<AddDimension>( "AddDimension" );
    CheckClass<RemoveDimension>( "RemoveDimension" );
    CheckClass<Modulus>( "Modulus" );
    CheckClass<DomainRotatePlane>( "DomainRotatePlane" );
    CHECK( Metadata::GetAll().size() == 47 );
    for( size_t i = 0; i < Metadata::GetAll().size(); i++ )
    {
        CHECK( Metadata::GetAll()[i]->id == i );
    }

    // DynamicCast to the wrong class is null (reference tests/FastNoiseCpp11Include.cpp:28-45)
    SmartNode<> base = New<Checkerboard>();
    CHECK( !SmartNode<Simplex>::DynamicCast( base ) );
    CHECK( SmartNode<ScalableGenerator>::DynamicCast( base ) );

    // a domain warp fractal takes only domain warp sources: the typed setter does not compile
    // for others, and the metadata setter refuses them
    auto warpFractal = New<DomainWarpFractalIndependent>();
    const Metadata& wfMeta = warpFractal->GetMetadata();
    CHECK( !wfMeta.memberNodeLookups[0].setFunc( warpFractal.get(), New<Simplex>() ) );
    CHECK( wfMeta.memberNodeLookups[0].setFunc( warpFractal.get(), New<DomainWarpSimplex>() ) );
    // setters of another node type refuse
    CHECK( !wfMeta.memberVariables[0].setFunc( New<Simplex>().get(), Metadata::MemberVariable::ValueUnion( 4 ) ) );

    // member formatting
    CHECK( Metadata::FormatMetadataNodeName( &Metadata::Get<DomainWarpFractalProgressive>() ) ==
           "Domain Warp Fractal Progressive" );
    CHECK( Metadata::FormatMetadataMemberName( Metadata::Get<DomainOffset>().memberHybrids[1] ) == "Y Offset" );

    // setters change exactly the members they name: the encoded tree shows them
    auto simplex = New<Simplex>();
    std::string plain = Encode( simplex.get() );
    simplex->SetScale( 50.0f );
    simplex->SetSeedOffset( 3 );
    simplex->SetOutputMin( -2.0f );
    simplex->SetOutputMax( 4.0f );
    std::string set = Encode( simplex.get() );
    CHECK( plain != set );
    {
        std::vector<std::unique_ptr<NodeData>> nodes;
        NodeData* data = Metadata::DeserialiseNodeData( set.c_str(), nodes );
        CHECK( data && data->metadata == &Metadata::Get<Simplex>() );
        if( data )
        {
            CHECK( data->variables[0].f == 50.0f );
            CHECK( data->variables[1].i == 3 );
            CHECK( data->variables[2].f == -2.0f );
            CHECK( data->variables[3].f == 4.0f );
            CHECK( Metadata::SerialiseNodeData( data ) == set );
        }
    }

    // the workload trees: encode -> NodeData -> encode is the identity, and the decoded tree
    // encodes to the same string
    SmartNode<> trees[] = { SimplexC0(), FbmPerlinC1(), TerrainC2(), BlendTree() };
    for( auto& tree : trees )
    {
        std::string enc = Encode( tree.get() );
        CHECK( !enc.empty() );
        std::vector<std::unique_ptr<NodeData>> nodes;
        NodeData* data = Metadata::DeserialiseNodeData( enc.c_str(), nodes );
        CHECK( data );
        if( data )
        {
            CHECK( Metadata::SerialiseNodeData( data ) == enc );
            CHECK( Metadata::SerialiseNodeData( data, true ) == enc );
        }
        SmartNode<> decoded = NewFromEncodedNodeTree( enc.c_str() );
        CHECK( decoded && Encode( decoded.get() ) == enc );
        CHECK( std::strcmp( decoded->GetMetadata().name, tree->GetMetadata().name ) == 0 );
    }

    // NodeData built by hand, with a node shared by two inputs (encoded once, referenced after)
    {
        std::vector<std::unique_ptr<NodeData>> own;
        own.emplace_back( new NodeData( &Metadata::Get<Simplex>() ) );
        NodeData* shared = own.back().get();
        own.emplace_back( new NodeData( &Metadata::Get<Add>() ) );
        NodeData* add = own.back().get();
        add->nodeLookups[0] = shared;
        add->hybrids[0].first = shared;
        std::string enc = Metadata::SerialiseNodeData( add );
        CHECK( !enc.empty() );
        SmartNode<> decoded = NewFromEncodedNodeTree( enc.c_str() );
        CHECK( decoded && std::strcmp( decoded->GetMetadata().name, "Add" ) == 0 );
        std::vector<std::unique_ptr<NodeData>> back;
        NodeData* again = Metadata::DeserialiseNodeData( enc.c_str(), back );
        CHECK( again && again->nodeLookups[0] && again->nodeLookups[0] == again->hybrids[0].first );

        // a loop: refused without fixUp; with fixUp the looping link is cut and the now unset
        // source makes the tree unencodable, as in the reference
        own.emplace_back( new NodeData( &Metadata::Get<FractalFBm>() ) );
        NodeData* fbm = own.back().get();
        own.emplace_back( new NodeData( &Metadata::Get<Abs>() ) );
        NodeData* abs = own.back().get();
        fbm->nodeLookups[0] = abs;
        abs->nodeLookups[0] = fbm;
        CHECK( Metadata::SerialiseNodeData( fbm ).empty() );
        CHECK( Metadata::SerialiseNodeData( fbm, true ).empty() );
        CHECK( abs->nodeLookups[0] == nullptr );
    }

    // invalid strings
    CHECK( !NewFromEncodedNodeTree( "not a tree" ) );
    CHECK( !NewFromEncodedNodeTree( nullptr ) );
    std::vector<std::unique_ptr<NodeData>> none;
    CHECK( Metadata::DeserialiseNodeData( "@@@@", none ) == nullptr );

    SmartNodeManager::SetMemoryPoolSize( 1 << 20 );
    std::printf( "meta: %d failures\n", g_failures );
    return g_failures ? 1 : 0;
}

static int EncodeTrees()
{
    SmartNode<> trees[] = { SimplexC0(), FbmPerlinC1(), TerrainC2(), BlendTree() };
    for( auto& tree : trees )
    {
        std::printf( "%s\n", Encode( tree.get() ).c_str() );
    }
    return 0;
}

// ---- gen ----

static bool WriteResult( const std::string& dir, const std::string& name, const std::vector<float>& values, OutputMinMax mm )
{
    FILE* f = std::fopen( ( dir + "/" + name + ".f32" ).c_str(), "wb" );
    if( !f ) return false;
    bool ok = std::fwrite( values.data(), sizeof( float ), values.size(), f ) == values.size();
    std::fclose( f );
    f = std::fopen( ( dir + "/" + name + ".mm" ).c_str(), "wb" );
    if( !f ) return false;
    float m[2] = { mm.min, mm.max };
    ok = ok && std::fwrite( m, sizeof( float ), 2, f ) == 2;
    std::fclose( f );
    return ok;
}

static int Gen( const std::string& dir )
{
    struct Job
    {
        const char* name;
        SmartNode<> tree;
    };
    Job jobs[] = { { "simplex_c0", SimplexC0() }, { "fbm_perlin_c1", FbmPerlinC1() }, { "terrain_c2", TerrainC2() },
                   { "blend_tree", BlendTree() } };
    for( auto& job : jobs )
    {
        // the same tree again, decoded from its encoded string
        std::string enc = Encode( job.tree.get() );
        SmartNode<> decoded = NewFromEncodedNodeTree( enc.c_str() );
        CHECK( decoded );
        if( !decoded ) continue;
        const SmartNode<> versions[2] = { job.tree, decoded };
        for( int v = 0; v < 2; v++ )
        {
            const Generator& g = *versions[v];
            std::string tag = std::string( job.name ) + ( v ? "_decoded" : "_setters" );
            std::vector<float> out( 64 * 64 * 64 );
            OutputMinMax mm = g.GenUniformGrid3D( out.data(), -128.0f, -128.0f, -128.0f, 64, 64, 64, 1.0f, 1.0f, 1.0f, 1337 );
            CHECK( WriteResult( dir, tag + "_grid3d", out, mm ) );
            std::vector<float> tile( 192 * 160 );
            mm = g.GenTileable2D( tile.data(), 192, 160, 1.0f, 1.0f, 7 );
            CHECK( WriteResult( dir, tag + "_tileable", tile, mm ) );
            std::vector<float> grid2( 300 * 200 );
            mm = g.GenUniformGrid2D( grid2.data(), 10.5f, -3.25f, 300, 200, 0.5f, 2.0f, -42 );
            CHECK( WriteResult( dir, tag + "_grid2d", grid2, mm ) );
            std::vector<float> grid4( 12 * 10 * 8 * 6 );
            mm = g.GenUniformGrid4D( grid4.data(), 1, 2, 3, 4, 12, 10, 8, 6, 1, 1, 1, 1, 99 );
            CHECK( WriteResult( dir, tag + "_grid4d", grid4, mm ) );
            std::vector<float> xs( 5000 ), ys( 5000 ), zs( 5000 ), pos( 5000 );
            for( int i = 0; i < 5000; i++ )
            {
                xs[i] = i * 0.6f;                                // the reference benchmark's positions
                ys[i] = i * -1.3f;
                zs[i] = i * 0.25f + 7.0f;
            }
            mm = g.GenPositionArray3D( pos.data(), 5000, xs.data(), ys.data(), zs.data(), 0.5f, 0.25f, -1.0f, 2024 );
            CHECK( WriteResult( dir, tag + "_pos3d", pos, mm ) );
            std::vector<float> single( 1, g.GenSingle3D( 12.5f, -7.25f, 3.0f, 5 ) );
            OutputMinMax none;
            CHECK( WriteResult( dir, tag + "_single3d", single, none ) );
        }
    }
    std::printf( "gen: %d failures\n", g_failures );
    return g_failures ? 1 : 0;
}

// ---- threads ----

static int Threads( int n )
{
    fnSetAutoSpecialise( 2 );                              // a tree used twice on the interpreter is specialised
    SmartNode<> tree = TerrainC2();
    const int X = 48, Y = 40, Z = 24;
    std::vector<float> ref3( X * Y * Z ), refT( 96 * 64 );
    fnSetJitEnabled( 0 );
    OutputMinMax ref3mm = tree->GenUniformGrid3D( ref3.data(), 3, -5, 11, X, Y, Z, 1, 1, 1, 77 );
    OutputMinMax refTmm = tree->GenTileable2D( refT.data(), 96, 64, 1, 1, 78 );
    fnSetJitEnabled( 1 );
    std::atomic<int> mismatches{ 0 }, calls{ 0 };
    std::vector<std::thread> pool;
    for( int t = 0; t < n; t++ )
    {
        pool.emplace_back( [&, t]
        {
            std::vector<float> out3( X * Y * Z ), outT( 96 * 64 );
            for( int k = 0; k < 12; k++ )
            {
                if( ( k + t ) % 2 == 0 )
                {
                    OutputMinMax mm = tree->GenUniformGrid3D( out3.data(), 3, -5, 11, X, Y, Z, 1, 1, 1, 77 );
                    if( std::memcmp( out3.data(), ref3.data(), ref3.size() * 4 ) || std::memcmp( &mm, &ref3mm, 8 ) ) ++mismatches;
                }
                else
                {
                    OutputMinMax mm = tree->GenTileable2D( outT.data(), 96, 64, 1, 1, 78 );
                    if( std::memcmp( outT.data(), refT.data(), refT.size() * 4 ) || std::memcmp( &mm, &refTmm, 8 ) ) ++mismatches;
                }
                ++calls;
            }
        } );
    }
    for( auto& th : pool ) th.join();
    int waited = fnAutoSpecialiseWait( 60000 );
    int spec3 = fnJitIsSpecialised( tree->GetNodeHandle(), 3 );
    int spec4 = fnJitIsSpecialised( tree->GetNodeHandle(), 4 );
    // after the swap, every thread sees the specialised kernels with the same results
    std::vector<std::thread> pool2;
    for( int t = 0; t < n; t++ )
    {
        pool2.emplace_back( [&]
        {
            std::vector<float> out3( X * Y * Z );
            OutputMinMax mm = tree->GenUniformGrid3D( out3.data(), 3, -5, 11, X, Y, Z, 1, 1, 1, 77 );
            if( std::memcmp( out3.data(), ref3.data(), ref3.size() * 4 ) || std::memcmp( &mm, &ref3mm, 8 ) ) ++mismatches;
            ++calls;
        } );
    }
    for( auto& th : pool2 ) th.join();
    std::printf( "threads: %d calls, %d mismatches, wait %d, specialised 3D %d 4D %d, last error %d\n", calls.load(),
                 mismatches.load(), waited, spec3, spec4, fnGetLastError() );
    return ( mismatches == 0 && waited == FN_OK && spec3 == 1 && spec4 == 1 ) ? 0 : 1;
}

int main( int argc, char** argv )
{
    if( argc >= 2 && !std::strcmp( argv[1], "meta" ) ) return Meta();
    if( argc >= 2 && !std::strcmp( argv[1], "encode" ) ) return EncodeTrees();
    if( argc >= 3 && !std::strcmp( argv[1], "gen" ) ) return Gen( argv[2] );
    if( argc >= 3 && !std::strcmp( argv[1], "threads" ) ) return Threads( std::atoi( argv[2] ) );
    std::fprintf( stderr, "usage: %s meta | encode | gen DIR | threads N\n", argv[0] );
    return 2;
}
