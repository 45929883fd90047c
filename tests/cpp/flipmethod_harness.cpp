// Houdini-free harness that drives BoraGB300::FLIPMethod the way SOP_FlipWater drives
// Bora::FLIPMethod (houdini/source/SOP_FlipWater.cpp:119-137 grid and parameters,
// :282-292 initialize, :315-323 newParticle per input point, :362 advanceOneFrame).
//
//   harness [frames] [out.bin]
//
// Exit status 0 = the frames ran and the water fell under gravity. With out.bin the
// initial and final particle stores are written for a comparison with the oracle:
// int64 n0, n0 x 3 float world positions, n0 x 3 float world velocities (initial);
// int64 n, n x 3 float positions, n x 3 float velocities, n int32 initial indices
// (final). Every frame re-uploads the store, so the library's ids index that frame's
// input; the harness composes them into indices of the initial store.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "BoraFLIPMethod.hpp"

static bool write_store( std::FILE* f, const BoraGB300::Particles& pts, const std::vector<int32_t>* origin )
{
    const int64_t n = (int64_t)pts.size();
    bool ok = std::fwrite( &n, sizeof( n ), 1, f ) == 1;
    ok = ok && std::fwrite( pts.position.data(), sizeof( float ), 3 * n, f ) == (size_t)( 3 * n );
    ok = ok && std::fwrite( pts.velocity.data(), sizeof( float ), 3 * n, f ) == (size_t)( 3 * n );
    if( origin ) ok = ok && std::fwrite( origin->data(), sizeof( int32_t ), n, f ) == (size_t)n;
    return ok;
}

int main( int argc, char** argv )
{
    const int frames = argc > 1 ? std::atoi( argv[1] ) : 3;
    std::FILE* out = nullptr;
    if( argc > 2 && !( out = std::fopen( argv[2], "wb" ) ) )
    {
        std::fprintf( stderr, "cannot open %s\n", argv[2] );
        return 1;
    }
    const float voxelSize = 1.f / 32.f;
    const float gridmin[3] = { 0.f, 0.f, 0.f }, gridmax[3] = { 1.f, 1.f, 1.f };
    BoraGB300::FLIPMethod flip;
    flip.params.dt = 1.f / 24.f / 4.f;
    flip.params.voxelSize = voxelSize;
    flip.params.wallLevel = 2.f;
    flip.params.projIteration = 5000;
    try
    {
        flip.initialize( 32, 32, 32, gridmin, gridmax );
        BoraGB300::Particles pts;
        // a block of fluid, 8 particles per cell on a regular sub-lattice
        for( int k = 0; k < 32; ++k )
            for( int j = 0; j < 16; ++j )
                for( int i = 0; i < 12; ++i )
                    for( int s = 0; s < 8; ++s )
                    {
                        const float p[3] = { ( i + 0.25f + 0.5f * ( s & 1 ) ) * voxelSize,
                                             ( j + 0.25f + 0.5f * ( ( s >> 1 ) & 1 ) ) * voxelSize,
                                             ( k + 0.25f + 0.5f * ( s >> 2 ) ) * voxelSize };
                        const float v[3] = { 0.f, 0.f, 0.f };
                        flip.newParticle( pts, p, v );
                    }
        double y0 = 0.0;
        for( size_t i = 0; i < pts.size(); ++i ) y0 += pts.position[3 * i + 1];
        y0 /= (double)pts.size();
        std::vector<int32_t> origin( pts.size() );
        for( size_t i = 0; i < origin.size(); ++i ) origin[i] = (int32_t)i;
        if( out && !write_store( out, pts, nullptr ) ) return 1;
        for( int f = 0; f < frames; ++f )
        {
            const int st = flip.advanceOneFrame( pts );
            std::vector<int32_t> next( pts.size() );
            for( size_t i = 0; i < next.size(); ++i ) next[i] = origin[(size_t)pts.id[i]];
            origin.swap( next );
            const bora_flip_stats s = flip.stats();
            std::printf( "frame %d status %d particles %zu tiles %d iters %d rel %.3e maxdx %.3e\n", f, st, pts.size(),
                         s.active_tiles, s.solver_iterations, s.residual_rel, s.residual_max_dx );
        }
        double y1 = 0.0, vy = 0.0;
        for( size_t i = 0; i < pts.size(); ++i ) { y1 += pts.position[3 * i + 1]; vy += pts.velocity[3 * i + 1]; }
        y1 /= (double)pts.size();
        vy /= (double)pts.size();
        std::printf( "mean height %.5f -> %.5f, mean vy %.5f\n", y0, y1, vy );
        if( out )
        {
            const bool ok = write_store( out, pts, &origin );
            std::fclose( out );
            if( !ok ) return 1;
        }
        return ( y1 < y0 && vy < 0.0 && pts.size() > 0 ) ? 0 : 2;
    }
    catch( const BoraGB300::Error& e )
    {
        std::fprintf( stderr, "error: %s\n", e.what() );
        return 1;
    }
}
