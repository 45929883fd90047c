// Houdini-free harness that drives BoraGB300::FLIPMethod the way SOP_FlipWater drives
// Bora::FLIPMethod (houdini/source/SOP_FlipWater.cpp:119-137 grid and parameters,
// :282-292 initialize, :315-323 newParticle per input point, :362 advanceOneFrame).
// Exit status 0 = the frames ran and the water fell under gravity.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "BoraFLIPMethod.hpp"

int main( int argc, char** argv )
{
    const int frames = argc > 1 ? std::atoi( argv[1] ) : 3;
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
        for( int f = 0; f < frames; ++f )
        {
            const int st = flip.advanceOneFrame( pts );
            const bora_flip_stats s = flip.stats();
            std::printf( "frame %d status %d particles %zu tiles %d iters %d rel %.3e maxdx %.3e\n", f, st, pts.size(),
                         s.active_tiles, s.solver_iterations, s.residual_rel, s.residual_max_dx );
        }
        double y1 = 0.0, vy = 0.0;
        for( size_t i = 0; i < pts.size(); ++i ) { y1 += pts.position[3 * i + 1]; vy += pts.velocity[3 * i + 1]; }
        y1 /= (double)pts.size();
        vy /= (double)pts.size();
        std::printf( "mean height %.5f -> %.5f, mean vy %.5f\n", y0, y1, vy );
        return ( y1 < y0 && vy < 0.0 && pts.size() > 0 ) ? 0 : 2;
    }
    catch( const BoraGB300::Error& e )
    {
        std::fprintf( stderr, "error: %s\n", e.what() );
        return 1;
    }
}
