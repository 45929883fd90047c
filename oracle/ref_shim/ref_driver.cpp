// ORACLE INFRASTRUCTURE: a C entry layer around the reference's own Bora::FLIPMethod
// (base/header/FLIPMethod.h:13-126), compiled for the host from the reference's
// unmodified sources through the shim headers in this directory. Tests use it to
// generate golden vectors and to pin the CPU restatement in oracle/flip_oracle.cpp.
// It is never part of the product library.
//
// The driver follows the order of Houdini's SOP_FlipWater
// (houdini/source/SOP_FlipWater.cpp:122-137,282-292,315-323,362) minus the world/voxel
// transforms: callers hand particles over in voxel space and call advanceOneStep
// directly (base/source/FLIPMethod.cu:208-298), which is what one frame runs.
#include <cstdint>
#include <cstddef>
#include <map>
#include <set>
#include <list>
#include <stack>
#include <queue>
#include <cmath>
#include <cfloat>
#include <cstring>
#include <bitset>
#include <vector>
#include <string>
#include <atomic>
#include <fstream>
#include <iomanip>
#include <climits>
#include <cstdlib>
#include <iostream>
#include <sstream>
#include <iterator>
#include <numeric>
#include <algorithm>
#include <chrono>
#include <unordered_set>
#include <unordered_map>
#include <thread>
#include <memory>
#include <functional>
#include <sys/stat.h>
#include <sys/time.h>

// Tests read the solver's linear system and the kill mask, which FLIPMethod and
// FluidProjection keep private.
#define private public
#include "Bora.h"
#undef private

extern "C" {

typedef struct RefParams
{
    float extForce[3];
    int maxsubsteps;
    float dt;
    float wallLevel;
    int enableWaterTank;
    int enableCurl;
    float dampingBand;
    float voxelSize;
    float colVelScale;
    int ptsPerCell;
    float vortPresRate;
    float adjacencyUnder;
    int projIteration;
    int redistIteration;
} RefParams;

struct RefSim
{
    Bora::FLIPMethod flip;
    Bora::Particles pts;
    Bora::Grid grid;
    RefSim() : pts( Bora::kUnified ) {}
};

void* ref_create( int nx, int ny, int nz, const float* bmin, const float* bmax, const RefParams* p )
{
    RefSim* s = new RefSim();
    s->grid.initialize( (size_t)nx, (size_t)ny, (size_t)nz,
                        Bora::Vec3f( bmin[0], bmin[1], bmin[2] ), Bora::Vec3f( bmax[0], bmax[1], bmax[2] ) );
    Bora::FLIPMethod::Params& q = s->flip.params;
    q.extForce = Bora::Vec3f( p->extForce[0], p->extForce[1], p->extForce[2] );
    q.maxsubsteps = p->maxsubsteps;
    q.dt = p->dt;
    q.wallLevel = p->wallLevel;
    q.enableWaterTank = p->enableWaterTank != 0;
    q.enableCurl = p->enableCurl != 0;
    q.dampingBand = p->dampingBand;
    q.voxelSize = p->voxelSize;
    q.colVelScale = p->colVelScale;
    q.ptsPerCell = p->ptsPerCell;
    q.vortPresRate = p->vortPresRate;
    q.adjacencyUnder = p->adjacencyUnder;
    q.projIteration = p->projIteration;
    q.redistIteration = p->redistIteration;
    s->flip.initialize( s->grid );
    return s;
}

void ref_destroy( void* h ) { delete (RefSim*)h; }

void ref_set_boxes( void* h, int n, const float* boxes, float band )
{
    RefSim* s = (RefSim*)h;
    BoraColliderSet set;
    std::memset( &set, 0, sizeof( set ) );
    set.count = n < BORA_MAX_COLLIDERS ? n : BORA_MAX_COLLIDERS;
    set.band = band;
    for( int b = 0; b < set.count; ++b )
        for( int c = 0; c < 3; ++c )
        {
            set.box[b].lo[c] = boxes[b * 9 + c];
            set.box[b].hi[c] = boxes[b * 9 + 3 + c];
            set.box[b].vel[c] = boxes[b * 9 + 6 + c];
        }
    s->flip._collisions.setBoxes( set );
}

// Appends particles already in voxel space (FLIPMethod::newParticle, FLIPMethod.h:75-99).
void ref_add_particles( void* h, const float* pos, const float* vel, size_t n )
{
    RefSim* s = (RefSim*)h;
    for( size_t i = 0; i < n; ++i )
        s->flip.newParticle( s->pts, Bora::Vec3f( pos[3 * i], pos[3 * i + 1], pos[3 * i + 2] ),
                             Bora::Vec3f( vel[3 * i], vel[3 * i + 1], vel[3 * i + 2] ) );
}

// FLIPMethod::fillWaterTank (FLIPMethod.cu:407-478) on the reference's own code; the new
// particles are brought to voxel space as particlesToVoxel would (FLIPMethod.cu:499-514).
size_t ref_fill_water_tank( void* h )
{
    RefSim* s = (RefSim*)h;
    const size_t n0 = s->pts.position.size();
    s->flip.fillWaterTank( s->pts );
    const size_t n1 = s->pts.position.size();
    for( size_t i = n0; i < n1; ++i )
    {
        s->pts.position[i] = s->flip._grid.voxelPoint( s->pts.position[i] );
        s->pts.velocity[i] = s->flip._grid.voxelVector( s->pts.velocity[i] );
    }
    return n1 - n0;
}

void ref_step( void* h, float dt )
{
    RefSim* s = (RefSim*)h;
    if( s->pts.position.size() == 0 ) return;
    s->flip.advanceOneStep( s->pts, dt );
}

// FLIPMethod::postProcess (FLIPMethod.cu:300-405) on the reference's own code, in voxel
// space (advanceOneFrame calls it before particlesToWorld).
void ref_post_process( void* h )
{
    RefSim* s = (RefSim*)h;
    if( s->pts.position.size() == 0 ) return;
    s->flip.postProcess( s->pts );
}

// Particle vorticity and curvature (Particles::vorticity / ::curvature).
void ref_get_attributes( void* h, float* vort, float* curv )
{
    RefSim* s = (RefSim*)h;
    const size_t n = s->pts.position.size();
    for( size_t i = 0; i < n; ++i )
    {
        if( vort ) vort[i] = s->pts.vorticity[i];
        if( curv ) curv[i] = s->pts.curvature[i];
    }
}

size_t ref_num_particles( void* h ) { return ((RefSim*)h)->pts.position.size(); }

void ref_get_particles( void* h, float* pos, float* vel, float* adj )
{
    RefSim* s = (RefSim*)h;
    const size_t n = s->pts.position.size();
    for( size_t i = 0; i < n; ++i )
    {
        const Bora::Vec3f& p = s->pts.position[i];
        const Bora::Vec3f& v = s->pts.velocity[i];
        if( pos ) { pos[3 * i] = p.x; pos[3 * i + 1] = p.y; pos[3 * i + 2] = p.z; }
        if( vel ) { vel[3 * i] = v.x; vel[3 * i + 1] = v.y; vel[3 * i + 2] = v.z; }
        if( adj ) adj[i] = s->pts.adjacency[i];
    }
}

// Kill mask of the last step, in the particle order before compaction.
size_t ref_get_removed( void* h, uint8_t* out )
{
    RefSim* s = (RefSim*)h;
    const size_t n = s->flip._removedPts.size();
    if( out ) for( size_t i = 0; i < n; ++i ) out[i] = (uint8_t)s->flip._removedPts[i];
    return n;
}

// out: fx, fy, fz, block, frame nx, ny, nz, active tiles
void ref_frame_info( void* h, int64_t* out )
{
    RefSim* s = (RefSim*)h;
    Bora::SparseFrame* f = s->flip._frame;
    out[0] = f->_fx; out[1] = f->_fy; out[2] = f->_fz; out[3] = f->_block_res;
    out[4] = (int64_t)f->_grid.nx(); out[5] = (int64_t)f->_grid.ny(); out[6] = (int64_t)f->_grid.nz();
    out[7] = (int64_t)f->_coords.size();
}

void ref_grid_xform( void* h, float* out )
{
    RefSim* s = (RefSim*)h;
    const Bora::Grid& g = s->flip._grid;
    out[0] = g._translate.x; out[1] = g._translate.y; out[2] = g._translate.z;
    out[3] = g._scale.x; out[4] = g._scale.y; out[5] = g._scale.z;
    out[6] = s->flip._voxelWallLevel;
    const Bora::Vec3f& e = s->flip._voxelExtForce;
    out[7] = e.x; out[8] = e.y; out[9] = e.z;
}

void ref_get_tiles( void* h, int64_t* ijk )
{
    RefSim* s = (RefSim*)h;
    Bora::SparseFrame* f = s->flip._frame;
    for( size_t t = 0; t < f->_coords.size(); ++t )
    {
        ijk[3 * t] = (int64_t)f->_coords[t].i;
        ijk[3 * t + 1] = (int64_t)f->_coords[t].j;
        ijk[3 * t + 2] = (int64_t)f->_coords[t].k;
    }
}

// Tile-marker counts of the last rebuild (SparseFrame::_markers), one per tile.
void ref_get_markers( void* h, int32_t* out )
{
    RefSim* s = (RefSim*)h;
    Bora::SparseFrame* f = s->flip._frame;
    for( size_t t = 0; t < f->_markers.size(); ++t ) out[t] = f->_markers[t];
}

size_t ref_field_size( void* h ) { return ((RefSim*)h)->flip._sMassField.size(); }

// which: 0 mass, 1 surf(count), 2 pres, 3 velo (3 floats), 4 comp (3 floats), 5 mark (int64)
void ref_get_field( void* h, int which, void* out )
{
    RefSim* s = (RefSim*)h;
    Bora::FLIPMethod& f = s->flip;
    const size_t n = f._sMassField.size();
    float* o = (float*)out;
    switch( which )
    {
        case 0: for( size_t i = 0; i < n; ++i ) o[i] = f._sMassField[i]; break;
        case 1: for( size_t i = 0; i < n; ++i ) o[i] = f._sSurfField[i]; break;
        case 2: for( size_t i = 0; i < n; ++i ) o[i] = f._sPresField[i]; break;
        case 3: for( size_t i = 0; i < n; ++i ) { o[3 * i] = f._sVeloField[i].x; o[3 * i + 1] = f._sVeloField[i].y; o[3 * i + 2] = f._sVeloField[i].z; } break;
        case 4: for( size_t i = 0; i < n; ++i ) { o[3 * i] = f._sCompField[i].x; o[3 * i + 1] = f._sCompField[i].y; o[3 * i + 2] = f._sCompField[i].z; } break;
        case 5: { int64_t* m = (int64_t*)out; for( size_t i = 0; i < n; ++i ) m[i] = (int64_t)f._sMarkField[i]; } break;
        default: break;
    }
}

size_t ref_num_unknowns( void* h ) { return ((RefSim*)h)->flip._projection._b.size(); }

// The projected system of the last step: right-hand side, solution and the storage
// index of each unknown's cell (FluidProjection.cu:174-186,265-266).
void ref_get_system( void* h, float* b, float* x, int64_t* cells )
{
    RefSim* s = (RefSim*)h;
    Bora::FluidProjection& P = s->flip._projection;
    const size_t n = P._b.size();
    for( size_t i = 0; i < n; ++i )
    {
        if( b ) b[i] = P._b[i];
        if( x ) x[i] = P._x[i];
        if( cells ) cells[i] = (int64_t)P._fluidCellBuffer[i];
    }
}

}  // extern "C"
