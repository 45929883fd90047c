// BoraFLIPMethod.hpp - header-only C++ wrapper that gives the C ABI of bora_flip.h the
// shape of the reference's Bora::FLIPMethod (base/header/FLIPMethod.h:13-126), so that a
// caller written against FLIPMethod (Houdini's SOP_FlipWater,
// houdini/source/SOP_FlipWater.cpp:122-137, 282-292, 296-363) changes only its types.
//
//   reference                                  this wrapper
//   Bora::FLIPMethod::Params params            BoraGB300::FLIPMethod::Params params (same fields)
//   initialize( const Grid& )                  initialize( grid ) / initialize( nx,ny,nz,min,max )
//   newParticle( Particles&, p, v )            newParticle( Particles&, p, v )
//   advanceOneFrame( Particles& )              advanceOneFrame( Particles& )   (step + postProcess)
//   postProcess( Particles& )                  postProcess( Particles& )       (voxel space)
//   advanceOneStep( Particles&, dt )           advanceOneStep( Particles&, dt )   (voxel space)
//   particlesToVoxel / particlesToWorld        particlesToVoxel / particlesToWorld
//   updateCollisionSource( vdb, vdb )          updateCollisionSource( voxels, phi, vel, background )
//                                              (the grids' active voxels) or setColliders( boxes )
//   getGrid()                                  getGrid() -> bora_frame_info
//
// Differences a caller sees: particles live in a host store (BoraGB300::Particles) that
// is uploaded before and read back after each call, ids travel with the particles
// (the reference reorders particles without ids), and failures throw BoraGB300::Error
// with the library's status code instead of passing silently.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "bora_flip.h"

namespace BoraGB300
{

class Error : public std::runtime_error
{
  public:
    int status;
    Error( int st, const std::string& what )
        : std::runtime_error( what + ": " + bora_flip_status_string( st ) ), status( st )
    {
    }
};

inline int check( int st, const char* what )
{
    if( st < 0 ) throw Error( st, what );
    return st;
}

// Host particle store: the attributes FLIPMethod reads and writes
// (Bora::Particles position, velocity, adjacency, vorticity, curvature; FLIPMethod.h:75-99)
// plus an id.
struct Particles
{
    std::vector<float> position;   // x,y,z per particle
    std::vector<float> velocity;   // x,y,z per particle
    std::vector<float> adjacency;  // one per particle
    std::vector<float> vorticity;  // one per particle (postProcess)
    std::vector<float> curvature;  // one per particle (postProcess)
    std::vector<int32_t> id;
    size_t size() const { return position.size() / 3; }
    void clear()
    {
        position.clear(); velocity.clear(); adjacency.clear(); vorticity.clear(); curvature.clear(); id.clear();
    }
};

class FLIPMethod
{
  public:
    // Bora::FLIPMethod::Params (FLIPMethod.h:51-67), same names and defaults, plus the
    // solver controls that the reference hard-codes.
    struct Params
    {
        float extForce[3] = { 0.f, -9.80665f, 0.f };
        int maxsubsteps = 1;
        float dt = 1.f / 24.f;
        float wallLevel = -1e+30f;
        bool enableWaterTank = false;
        bool enableCurl = false;
        float dampingBand = 0.f;
        float voxelSize = 0.1f;
        float colVelScale = 1.f;
        int ptsPerCell = 8;
        float vortPresRate = 0.2f;
        float adjacencyUnder = 2.f;
        int projIteration = 200;
        int redistIteration = 80;
        int solver = BORA_SOLVER_PLAIN;
        double tolerance = 1e-6;
        double divTolerance = 1e-5;
        int advection = BORA_ADVECT_EULER;
        bool warmStart = false;  // start each pressure solve from the last step's pressure (bora_flip_params.warm_start)
    } params;

    FLIPMethod() = default;
    FLIPMethod( const FLIPMethod& ) = delete;
    FLIPMethod& operator=( const FLIPMethod& ) = delete;
    ~FLIPMethod()
    {
        if( _h ) bora_flip_destroy( _h );
    }

    // FLIPMethod::initialize (FLIPMethod.cu:16-47) from a resolution and a world box.
    void initialize( int nx, int ny, int nz, const float minp[3], const float maxp[3] )
    {
        if( _h ) { bora_flip_destroy( _h ); _h = nullptr; }
        bora_grid_desc g;
        g.nx = nx; g.ny = ny; g.nz = nz;
        for( int a = 0; a < 3; ++a ) { g.min[a] = minp[a]; g.max[a] = maxp[a]; }
        const bora_flip_params p = toC();
        check( bora_flip_create( &g, &p, &_h ), "bora_flip_create" );
        _frameCount = 0;
    }

    // From any grid type with nx()/ny()/nz() and boundingBox().minPoint()/maxPoint()
    // returning x/y/z members (Bora::Grid, base/header/Grid.h:212-262).
    template <class GridT> void initialize( const GridT& grid )
    {
        const auto box = grid.boundingBox();
        const auto lo = box.minPoint();
        const auto hi = box.maxPoint();
        const float mn[3] = { lo.x, lo.y, lo.z }, mx[3] = { hi.x, hi.y, hi.z };
        initialize( (int)grid.nx(), (int)grid.ny(), (int)grid.nz(), mn, mx );
    }

    // FLIPMethod::newParticle (FLIPMethod.h:75-99): append one particle to the host store.
    void newParticle( Particles& pts, const float p[3], const float v[3] ) const
    {
        for( int a = 0; a < 3; ++a ) { pts.position.push_back( p[a] ); pts.velocity.push_back( v[a] ); }
        pts.adjacency.push_back( 0.f );
        pts.vorticity.push_back( 0.f );
        pts.curvature.push_back( 0.f );
        pts.id.push_back( -1 );
    }

    // FLIPMethod::fillWaterTank (FLIPMethod.cu:407-478): append the tank's particles (world
    // space, zero velocity) below params.wallLevel to the host store.
    void fillWaterTank( Particles& pts )
    {
        requireInit();
        const bora_flip_params p = toC();
        check( bora_flip_set_params( _h, &p ), "bora_flip_set_params" );
        const size_t n = pts.size();
        if( pts.velocity.size() != 3 * n ) pts.velocity.resize( 3 * n, 0.f );
        check( bora_flip_set_particles( _h, pts.position.data(), pts.velocity.data(), n, BORA_SPACE_WORLD ),
               "bora_flip_set_particles" );
        check( bora_flip_fill_water_tank( _h, nullptr ), "bora_flip_fill_water_tank" );
        size_t m = 0;
        check( bora_flip_num_particles( _h, &m ), "bora_flip_num_particles" );
        pts.position.resize( 3 * m );
        pts.velocity.resize( 3 * m );
        pts.adjacency.resize( m );
        pts.id.resize( m );
        check( bora_flip_get_particles( _h, pts.position.data(), pts.velocity.data(), pts.adjacency.data(),
                                        pts.id.data(), m, &m, BORA_SPACE_WORLD ),
               "bora_flip_get_particles" );
    }

    // CollisionSource replacement: analytic boxes (lo xyz, hi xyz, velocity xyz; voxel units).
    void setColliders( const std::vector<float>& boxes, float band = 3.f )
    {
        requireInit();
        check( bora_flip_set_colliders( _h, boxes.data(), (int)( boxes.size() / 9 ), band ), "bora_flip_set_colliders" );
    }

    // FLIPMethod::updateCollisionSource (FLIPMethod.h:111-114 -> CollisionSource::update):
    // the collider level set's active voxels (frame cells, 3 ints each), their signed
    // distances (world units) and velocities (world units per second, may be empty), and
    // the level set's background (world units) - what OpenVDB's active-value iterator
    // yields after sampling the grids at the frame's cell centres.
    void updateCollisionSource( const std::vector<int32_t>& ijk, const std::vector<float>& phi,
                                const std::vector<float>& vel, float background )
    {
        requireInit();
        const size_t n = phi.size();
        if( ijk.size() != 3 * n || ( !vel.empty() && vel.size() != 3 * n ) )
            throw Error( BORA_ERR_INVALID_ARG, "updateCollisionSource" );
        check( bora_flip_set_collider_voxels( _h, ijk.data(), phi.data(), vel.empty() ? nullptr : vel.data(), n,
                                              background ),
               "bora_flip_set_collider_voxels" );
    }

    // FLIPMethod::advanceOneFrame (FLIPMethod.cu:177-206): world-space particles in, one
    // step of params.dt and postProcess, world-space particles out.
    int advanceOneFrame( Particles& pts )
    {
        if( pts.size() == 0 ) return BORA_OK;  // FLIPMethod.cu:179
        const int st = run( pts, params.dt, BORA_SPACE_WORLD, true, true );
        ++_frameCount;
        return st;
    }

    // FLIPMethod::advanceOneStep (FLIPMethod.cu:208-298): voxel-space particles.
    int advanceOneStep( Particles& pts, float dt ) { return run( pts, dt, BORA_SPACE_VOXEL, true, false ); }

    // FLIPMethod::postProcess (FLIPMethod.cu:300-405) on voxel-space particles: updates
    // their vorticity and curvature; the surface is then in the handle's fields
    // (BORA_FIELD_SURF over the active tiles, bora_flip_get_field).
    void postProcess( Particles& pts ) { run( pts, 0.f, BORA_SPACE_VOXEL, false, true ); }

    // FLIPMethod::particlesToVoxel / particlesToWorld (FLIPMethod.cu:481-513).
    void particlesToVoxel( Particles& pts ) const { transform( pts, true ); }
    void particlesToWorld( Particles& pts ) const { transform( pts, false ); }

    bora_frame_info getGrid() const
    {
        bora_frame_info f{};
        if( _h ) check( bora_flip_frame_info( _h, &f ), "bora_flip_frame_info" );
        return f;
    }

    bora_flip_stats stats() const
    {
        bora_flip_stats s{};
        if( _h ) check( bora_flip_get_stats( _h, &s ), "bora_flip_get_stats" );
        return s;
    }

    bora_flip_handle handle() const { return _h; }
    int currentFrame() const { return _frameCount; }

  private:
    bora_flip_handle _h = nullptr;
    int _frameCount = 0;

    void requireInit() const
    {
        if( !_h ) throw Error( BORA_ERR_INVALID_ARG, "FLIPMethod used before initialize()" );
    }

    bora_flip_params toC() const
    {
        bora_flip_params p;
        bora_flip_default_params( &p );
        for( int a = 0; a < 3; ++a ) p.ext_force[a] = params.extForce[a];
        p.max_substeps = params.maxsubsteps;
        p.dt = params.dt;
        p.wall_level = params.wallLevel;
        p.enable_water_tank = params.enableWaterTank ? 1 : 0;
        p.enable_curl = params.enableCurl ? 1 : 0;
        p.damping_band = params.dampingBand;
        p.voxel_size = params.voxelSize;
        p.col_vel_scale = params.colVelScale;
        p.pts_per_cell = params.ptsPerCell;
        p.vort_pres_rate = params.vortPresRate;
        p.adjacency_under = params.adjacencyUnder;
        p.proj_iteration = params.projIteration;
        p.redist_iteration = params.redistIteration;
        p.solver = params.solver;
        p.tolerance = params.tolerance;
        p.div_tolerance = params.divTolerance;
        p.advection = params.advection;
        p.warm_start = params.warmStart ? 1 : 0;
        return p;
    }

    int run( Particles& pts, float dt, int space, bool step, bool post )
    {
        requireInit();
        const bora_flip_params p = toC();
        check( bora_flip_set_params( _h, &p ), "bora_flip_set_params" );
        const size_t n = pts.size();
        if( pts.velocity.size() != 3 * n ) pts.velocity.resize( 3 * n, 0.f );
        check( bora_flip_set_particles( _h, pts.position.data(), pts.velocity.data(), n, space ), "bora_flip_set_particles" );
        const bool attrs = pts.vorticity.size() == n && pts.curvature.size() == n;
        if( attrs && n )
            check( bora_flip_set_particle_attributes( _h, pts.vorticity.data(), pts.curvature.data(), n ),
                   "bora_flip_set_particle_attributes" );
        const int st = step ? check( bora_flip_step( _h, dt ), "bora_flip_step" ) : BORA_OK;
        if( post ) check( bora_flip_post_process( _h ), "bora_flip_post_process" );
        size_t m = 0;
        check( bora_flip_num_particles( _h, &m ), "bora_flip_num_particles" );
        pts.position.resize( 3 * m );
        pts.velocity.resize( 3 * m );
        pts.adjacency.resize( m );
        pts.id.resize( m );
        check( bora_flip_get_particles( _h, pts.position.data(), pts.velocity.data(), pts.adjacency.data(),
                                        pts.id.data(), m, &m, space ),
               "bora_flip_get_particles" );
        if( attrs || post )
        {
            pts.vorticity.resize( m );
            pts.curvature.resize( m );
            check( bora_flip_get_particle_attributes( _h, pts.vorticity.data(), pts.curvature.data(), nullptr, m, &m ),
                   "bora_flip_get_particle_attributes" );
        }
        return st;
    }

    void transform( Particles& pts, bool toVoxel ) const
    {
        const bora_frame_info f = getGrid();
        for( size_t i = 0; i < pts.size(); ++i )
            for( int a = 0; a < 3; ++a )
            {
                float& x = pts.position[3 * i + a];
                float& v = pts.velocity[3 * i + a];
                if( toVoxel ) { x = ( x - f.translate[a] ) / f.scale[a]; v = v / f.scale[a]; }
                else { x = x * f.scale[a] + f.translate[a]; v = v * f.scale[a]; }
            }
    }
};

}  // namespace BoraGB300
