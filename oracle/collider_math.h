/* ORACLE INFRASTRUCTURE: analytic box colliders sampled at cell centres.
 *
 * The reference ingests an OpenVDB level set and velocity grid into sparse fields of
 * cell-centre samples and queries them by trilinear lerp
 * (base/header/CollisionSource.h:66-150). OpenVDB is not available, so colliders are
 * restated as analytic boxes whose cell-centre samples are computed on the fly:
 *   phi(c)  = min over boxes of the box signed distance at the cell centre c (voxel
 *             units), clamped to [-band, band] (a level set outside its narrow band
 *             reads +/- its background value);
 *   vel(c)  = velocity of the box that attains the minimum when phi(c) < band, else 0;
 *   nrm(c)  = central-difference gradient of the clamped phi at c (neighbour indices
 *             clamped to the grid), normalised like Vec3f::normalized()
 *             (base/header/Vector3.h:350-354).
 * Queries use SparseField::lerp's rule (base/header/SparseField.h:150-173).
 *
 * A sparse collider (CollisionSource::update, CollisionSource.h:66-126, from a level set's
 * active voxels) replaces the boxes when tslot is set: the collider's 8^3 tiles over the
 * frame's tile grid hold cell-centre samples (phi, velocity; voxel units); cells outside
 * them read the background phi with zero velocity and zero normal (the reference's
 * fields' backgrounds outside the collider frame); normals on the collider's tiles are the
 * same normalised central differences of phi.
 * Shared by the CPU oracle restatement and the reference host shim so that both read
 * identical collider samples. Compile without floating-point contraction. */
#ifndef BORA_COLLIDER_MATH_H
#define BORA_COLLIDER_MATH_H

#include <math.h>

#define BORA_MAX_COLLIDERS 8
#define BORA_COLLIDER_PHI 0
#define BORA_COLLIDER_NORMAL 1
#define BORA_COLLIDER_VELOCITY 2

typedef struct BoraColliderBox
{
    float lo[3];
    float hi[3];
    float vel[3];
} BoraColliderBox;

typedef struct BoraColliderSet
{
    int count;
    float band;
    BoraColliderBox box[BORA_MAX_COLLIDERS];
    /* sparse collider: tile slot table over the frame's 8^3 tile grid (or NULL), samples */
    const int* tslot;
    const float* tphi;  /* [slots * 512] */
    const float* tvel;  /* [slots * 512 * 3] or NULL (zero) */
    float tbg;
    int ttx, tty;
} BoraColliderSet;

static inline int bora_collider_active( const BoraColliderSet* s ) { return s->count > 0 || s->tslot != 0; }

/* the sparse collider's slot of the tile holding cell (i,j,k), or -1 */
static inline int bora_collider_tile_slot( const BoraColliderSet* s, int i, int j, int k )
{
    return s->tslot[(size_t)( i >> 3 ) + (size_t)s->ttx * ( (size_t)( j >> 3 ) + (size_t)s->tty * (size_t)( k >> 3 ) )];
}
static inline size_t bora_collider_local( int i, int j, int k )
{
    return (size_t)( ( i & 7 ) | ( ( j & 7 ) << 3 ) | ( ( k & 7 ) << 6 ) );
}

static inline float bora_box_sdf( const BoraColliderBox* b, float px, float py, float pz )
{
    const float cx = ( b->lo[0] + b->hi[0] ) * 0.5f;
    const float cy = ( b->lo[1] + b->hi[1] ) * 0.5f;
    const float cz = ( b->lo[2] + b->hi[2] ) * 0.5f;
    const float hx = ( b->hi[0] - b->lo[0] ) * 0.5f;
    const float hy = ( b->hi[1] - b->lo[1] ) * 0.5f;
    const float hz = ( b->hi[2] - b->lo[2] ) * 0.5f;
    const float qx = fabsf( px - cx ) - hx;
    const float qy = fabsf( py - cy ) - hy;
    const float qz = fabsf( pz - cz ) - hz;
    const float ox = qx > 0.f ? qx : 0.f;
    const float oy = qy > 0.f ? qy : 0.f;
    const float oz = qz > 0.f ? qz : 0.f;
    const float outside = sqrtf( ox * ox + oy * oy + oz * oz );
    float m = qx > qy ? qx : qy;
    m = m > qz ? m : qz;
    const float inside = m < 0.f ? m : 0.f;
    return outside + inside;
}

/* Clamped phi sample at cell (i,j,k); *arg receives the index of the closest box. */
static inline float bora_collider_phi_cell( const BoraColliderSet* s, int i, int j, int k, int* arg )
{
    if( s->tslot )
    {
        const int sl = bora_collider_tile_slot( s, i, j, k );
        if( arg ) *arg = 0;
        return sl < 0 ? s->tbg : s->tphi[(size_t)sl * 512 + bora_collider_local( i, j, k )];
    }
    const float px = (float)i + 0.5f, py = (float)j + 0.5f, pz = (float)k + 0.5f;
    float best = s->band;
    int a = -1;
    for( int n = 0; n < s->count; ++n )
    {
        const float d = bora_box_sdf( &s->box[n], px, py, pz );
        if( a < 0 || d < best ) { best = d; a = n; }
    }
    if( best > s->band ) best = s->band;
    if( best < -s->band ) best = -s->band;
    if( arg ) *arg = a;
    return best;
}

static inline void bora_collider_sample( const BoraColliderSet* s, int nx, int ny, int nz,
                                         int i, int j, int k, int which, float out[3] )
{
    int a;
    if( which == BORA_COLLIDER_PHI )
    {
        out[0] = bora_collider_phi_cell( s, i, j, k, &a );
        out[1] = out[2] = 0.f;
        return;
    }
    if( s->tslot && which == BORA_COLLIDER_VELOCITY )
    {
        const int sl = bora_collider_tile_slot( s, i, j, k );
        const size_t c = (size_t)sl * 512 + bora_collider_local( i, j, k );
        const int have = sl >= 0 && s->tvel;
        out[0] = have ? s->tvel[3 * c] : 0.f;
        out[1] = have ? s->tvel[3 * c + 1] : 0.f;
        out[2] = have ? s->tvel[3 * c + 2] : 0.f;
        return;
    }
    if( s->tslot && bora_collider_tile_slot( s, i, j, k ) < 0 )
    {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    if( which == BORA_COLLIDER_VELOCITY )
    {
        const float phi = bora_collider_phi_cell( s, i, j, k, &a );
        if( a >= 0 && phi < s->band )
        {
            out[0] = s->box[a].vel[0];
            out[1] = s->box[a].vel[1];
            out[2] = s->box[a].vel[2];
        }
        else
        {
            out[0] = out[1] = out[2] = 0.f;
        }
        return;
    }
    {
        const int i0 = i > 0 ? i - 1 : 0, i1 = i < nx - 1 ? i + 1 : nx - 1;
        const int j0 = j > 0 ? j - 1 : 0, j1 = j < ny - 1 ? j + 1 : ny - 1;
        const int k0 = k > 0 ? k - 1 : 0, k1 = k < nz - 1 ? k + 1 : nz - 1;
        const float gx = ( bora_collider_phi_cell( s, i1, j, k, 0 ) - bora_collider_phi_cell( s, i0, j, k, 0 ) ) * 0.5f;
        const float gy = ( bora_collider_phi_cell( s, i, j1, k, 0 ) - bora_collider_phi_cell( s, i, j0, k, 0 ) ) * 0.5f;
        const float gz = ( bora_collider_phi_cell( s, i, j, k1, 0 ) - bora_collider_phi_cell( s, i, j, k0, 0 ) ) * 0.5f;
        const double d = 1.0f / sqrtf( gx * gx + gy * gy + gz * gz + 1e-30f );
        out[0] = (float)( gx * d );
        out[1] = (float)( gy * d );
        out[2] = (float)( gz * d );
    }
}

static inline int bora_clampi( int x, int lo, int hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }
static inline float bora_clampf( float x, float lo, float hi ) { return x < lo ? lo : ( x > hi ? hi : x ); }

/* SparseField::lerp (base/header/SparseField.h:150-173) over the collider samples. */
static inline void bora_collider_lerp( const BoraColliderSet* s, int nx, int ny, int nz,
                                       float px, float py, float pz, int which, float out[3] )
{
    const int i = bora_clampi( (int)( px - 0.5f ), 0, nx - 2 );
    const int j = bora_clampi( (int)( py - 0.5f ), 0, ny - 2 );
    const int k = bora_clampi( (int)( pz - 0.5f ), 0, nz - 2 );
    const float x = bora_clampf( px - ( (float)i + 0.5f ), 0.f, 1.f );
    const float y = bora_clampf( py - ( (float)j + 0.5f ), 0.f, 1.f );
    const float z = bora_clampf( pz - ( (float)k + 0.5f ), 0.f, 1.f );
    float f000[3], f100[3], f001[3], f101[3], f010[3], f110[3], f011[3], f111[3];
    bora_collider_sample( s, nx, ny, nz, i, j, k, which, f000 );
    bora_collider_sample( s, nx, ny, nz, i + 1, j, k, which, f100 );
    bora_collider_sample( s, nx, ny, nz, i, j, k + 1, which, f001 );
    bora_collider_sample( s, nx, ny, nz, i + 1, j, k + 1, which, f101 );
    bora_collider_sample( s, nx, ny, nz, i, j + 1, k, which, f010 );
    bora_collider_sample( s, nx, ny, nz, i + 1, j + 1, k, which, f110 );
    bora_collider_sample( s, nx, ny, nz, i, j + 1, k + 1, which, f011 );
    bora_collider_sample( s, nx, ny, nz, i + 1, j + 1, k + 1, which, f111 );
    for( int c = 0; c < 3; ++c )
    {
        const float c00 = f000[c] * ( 1.f - x ) + f100[c] * x;
        const float c01 = f001[c] * ( 1.f - x ) + f101[c] * x;
        const float c10 = f010[c] * ( 1.f - x ) + f110[c] * x;
        const float c11 = f011[c] * ( 1.f - x ) + f111[c] * x;
        const float c0 = c00 * ( 1.f - y ) + c10 * y;
        const float c1 = c01 * ( 1.f - y ) + c11 * y;
        out[c] = c0 * ( 1.f - z ) + c1 * z;
    }
}

#endif
