// Sparse field -> VDB conversion on the device, as 8^3 leaf blocks.
//
// The Houdini node turns the surface and velocity fields into OpenVDB grids after every
// frame (houdini/source/SOP_FlipWater.cpp:252-264) with FieldCast's convertSurfaceVDB
// (base/header/FieldCast.h:362-440) and convertVelocityVDB (:14-48). OpenVDB's leaf nodes
// are 8^3 voxel blocks at multiples of 8, exactly the frame's tiles (VDB voxel (i,j,k) =
// frame cell (i,j,k), transform: voxel size dx, translate min + dx/2), so the conversion
// here writes one leaf per tile - origin, 512-bit active mask and 512 values - and a caller
// that has OpenVDB copies leaves straight into a tree:
//   surface:  value = phi * dx over the cells of active tiles inside the grid (active),
//             background * dx elsewhere (inactive); with the water tank on, every voxel of
//             the 3-cell border band (below the grid, and around its sides up to 3 cells
//             above the water level) becomes active with min(cell centre y - level, value)
//             (FieldCast.h:398-440), which adds the leaves of the band outside the tiles;
//   velocity: value = v * dx (Grid::worldVector) over the cells of active tiles inside the
//             grid, active unless |v| < 1e-30 (FieldCast.h:33-45), 0 elsewhere.
// The float arithmetic follows FieldCast's operation order (this unit is compiled without
// floating-point contraction).
#include <algorithm>
#include <vector>

#include "bora_internal.h"

namespace {

struct VdbBand
{
    int on;            // water tank
    int ei, ek;        // last cell index per axis (grid nx - 1, nz - 1)
    int lv;            // int( (level - min.y) / dx + 1 )
    float level;       // water level (world)
    float ty, sy;      // world transform in y: y = j' * sy + ty for voxel coordinate j'
};

// FieldCast.h:408-438: the five slabs of the band (3 cells wide)
__device__ inline bool in_band( const VdbBand& b, int i, int j, int k )
{
    constexpr int bnd = 3;
    const bool ik_all = i >= -bnd && i <= b.ei + bnd && k >= -bnd && k <= b.ek + bnd;
    if( !ik_all || j < -bnd ) return false;
    if( j <= 0 ) return true;                  // below / at the grid bottom
    if( j > b.lv + bnd ) return false;
    return i <= 0 || i >= b.ei || k <= 0 || k >= b.ek;  // the four side walls
}

// One CTA per leaf, one thread per voxel (x fastest). leaf_slot: the tile's slot, or -1 for
// a band leaf outside the active tiles.
__global__ void __launch_bounds__( 512 ) k_vdb_surface( int nx, int ny, int nz, const int32_t* __restrict__ leaf_ijk,
                                                        const int32_t* __restrict__ leaf_slot,
                                                        const float* __restrict__ surf, float dx, float bg,
                                                        VdbBand band, uint64_t* __restrict__ mask,
                                                        float* __restrict__ val )
{
    const int leaf = blockIdx.x, l = threadIdx.x;
    const int i = leaf_ijk[3 * leaf] + ( l & 7 ), j = leaf_ijk[3 * leaf + 1] + ( ( l >> 3 ) & 7 ),
              k = leaf_ijk[3 * leaf + 2] + ( l >> 6 );
    const int slot = leaf_slot[leaf];
    float v = bg * dx;
    bool act = false;
    if( slot >= 0 && i >= 0 && j >= 0 && k >= 0 && i < nx && j < ny && k < nz )
    {
        v = surf[(size_t)slot * BORA_TILE_CELLS + l] * dx;
        act = true;
    }
    if( band.on && in_band( band, i, j, k ) )
    {
        const float cy = ( (float)j + 0.5f ) * band.sy + band.ty;  // Grid::worldPoint
        const float a = cy - band.level;
        v = a < v ? a : v;  // Min
        act = true;
    }
    val[(size_t)leaf * 512 + l] = v;
    const unsigned bits = __ballot_sync( 0xffffffffu, act );
    if( ( l & 31 ) == 0 ) reinterpret_cast<uint32_t*>( mask + (size_t)leaf * 8 )[l >> 5] = bits;
}

__global__ void __launch_bounds__( 512 ) k_vdb_velocity( int nx, int ny, int nz, const int32_t* __restrict__ leaf_ijk,
                                                         const int32_t* __restrict__ leaf_slot,
                                                         const float* __restrict__ vx, const float* __restrict__ vy,
                                                         const float* __restrict__ vz, float3 scale,
                                                         uint64_t* __restrict__ mask, float* __restrict__ val )
{
    const int leaf = blockIdx.x, l = threadIdx.x;
    const int i = leaf_ijk[3 * leaf] + ( l & 7 ), j = leaf_ijk[3 * leaf + 1] + ( ( l >> 3 ) & 7 ),
              k = leaf_ijk[3 * leaf + 2] + ( l >> 6 );
    const int slot = leaf_slot[leaf];
    float wx = 0.f, wy = 0.f, wz = 0.f;
    bool act = false;
    if( slot >= 0 && i < nx && j < ny && k < nz )
    {
        const size_t c = (size_t)slot * BORA_TILE_CELLS + l;
        wx = vx[c] * scale.x;  // Grid::worldVector
        wy = vy[c] * scale.y;
        wz = vz[c] * scale.z;
        act = !( sqrtf( wx * wx + wy * wy + wz * wz ) < 1e-30f );  // Vec3f::length
        if( !act ) wx = wy = wz = 0.f;
    }
    float* o = val + ( (size_t)leaf * 512 + l ) * 3;
    o[0] = wx;
    o[1] = wy;
    o[2] = wz;
    const unsigned bits = __ballot_sync( 0xffffffffu, act );
    if( ( l & 31 ) == 0 ) reinterpret_cast<uint32_t*>( mask + (size_t)leaf * 8 )[l >> 5] = bits;
}

}  // namespace

// FieldCast.h:404, int lv = (waterlevel - min.y) / dx + 1, with the float kept inside int range
int bora_vdb_level_index( float level, float min_y, float dx )
{
    const float f = ( level - min_y ) / dx + 1.f;
    return (int)std::max( -1.0e9f, std::min( 1.0e9f, f ) );
}

void bora_launch_vdb_surface( const BoraGridDev& g, const float* scale, const float* translate, int nleaves,
                              const int32_t* leaf_ijk, const int32_t* leaf_slot, const float* surf, float bg, int tank,
                              float level, uint64_t* mask, float* val, cudaStream_t st )
{
    if( nleaves <= 0 ) return;
    const float dx = scale[0];
    VdbBand b{};
    b.on = tank;
    b.ei = g.nx - 1;
    b.ek = g.nz - 1;
    b.lv = bora_vdb_level_index( level, translate[1], dx );
    b.level = level;
    b.ty = translate[1];
    b.sy = scale[1];
    k_vdb_surface<<<nleaves, 512, 0, st>>>( g.nx, g.ny, g.nz, leaf_ijk, leaf_slot, surf, dx, bg, b, mask, val );
}

void bora_launch_vdb_velocity( const BoraGridDev& g, const float* scale, int nleaves, const int32_t* leaf_ijk,
                               const int32_t* leaf_slot, const float* vx, const float* vy, const float* vz,
                               uint64_t* mask, float* val, cudaStream_t st )
{
    if( nleaves <= 0 ) return;
    k_vdb_velocity<<<nleaves, 512, 0, st>>>( g.nx, g.ny, g.nz, leaf_ijk, leaf_slot, vx, vy, vz,
                                             make_float3( scale[0], scale[1], scale[2] ), mask, val );
}

// The band's leaves (tile coordinates, possibly -1 or one past the tile grid) for the
// water tank with level `level`: every tile that holds a voxel of the band.
void bora_vdb_band_tiles( const BoraGridDev& g, const float* scale, const float* translate, float level,
                          std::vector<int32_t>& tiles )
{
    const float dx = scale[0];
    const int ei = g.nx - 1, ek = g.nz - 1;
    const int lv = bora_vdb_level_index( level, translate[1], dx );
    constexpr int bnd = 3;
    auto tile_of = []( int c ) { return c >= 0 ? c / 8 : -( ( -c + 7 ) / 8 ); };
    const int ti0 = tile_of( -bnd ), ti1 = tile_of( ei + bnd ), tk0 = tile_of( -bnd ), tk1 = tile_of( ek + bnd );
    const int tj0 = tile_of( -bnd ), tj1 = tile_of( std::max( 0, lv + bnd ) );
    for( int tk = tk0; tk <= tk1; ++tk )
        for( int tj = tj0; tj <= tj1; ++tj )
            for( int ti = ti0; ti <= ti1; ++ti )
            {
                // does the tile hold a band voxel? (the band is a union of boxes)
                const int i0 = ti * 8, j0 = tj * 8, k0 = tk * 8;
                const int i1 = i0 + 7, j1 = j0 + 7, k1 = k0 + 7;
                auto overlap = [&]( int a0, int a1, int b0, int b1 ) { return a0 <= b1 && b0 <= a1; };
                const bool ik = overlap( i0, i1, -bnd, ei + bnd ) && overlap( k0, k1, -bnd, ek + bnd );
                if( !ik ) continue;
                bool hit = overlap( j0, j1, -bnd, 0 );
                if( !hit && overlap( j0, j1, -bnd, lv + bnd ) )
                    hit = overlap( i0, i1, -bnd, 0 ) || overlap( i0, i1, ei, ei + bnd ) || overlap( k0, k1, -bnd, 0 ) ||
                          overlap( k0, k1, ek, ek + bnd );
                if( hit )
                {
                    tiles.push_back( ti );
                    tiles.push_back( tj );
                    tiles.push_back( tk );
                }
            }
}
