// ORACLE INFRASTRUCTURE: stand-in for the reference's CollisionSource
// (base/header/CollisionSource.h). The reference samples an OpenVDB level set and
// velocity grid into its own sparse fields (CollisionSource.h:66-126, host-only,
// needs OpenVDB, which is not available) and answers queries by trilinear lerp of the
// samples with a background value outside the sampled tiles (CollisionSource.h:128-150).
//
// This stand-in keeps the query semantics and replaces the ingest by analytic boxes:
//   * with no collider (the reference's "no input" case) signedDistance() returns the
//     background 5 and normal()/velocity() return zero (CollisionSource.h:56-58,130);
//   * with boxes, the cell-centre samples come from collider_math.h (shared with the
//     CPU oracle restatement) and are interpolated with SparseField::lerp's rule
//     (base/header/SparseField.h:150-173).
#pragma once

#include "collider_math.h"

BORA_NAMESPACE_BEGIN

class CollisionSource
{
    public:

        Grid _grid;
        BoraColliderSet _set;

    public:

        void initialize( const Grid& inGrid, const bool useCurve=false )
        {
            (void)useCurve;
            SparseFrame* f = SparseFrame::create( inGrid, kUnified );
            _grid = f->_grid;
            SparseFrame::remove( f );
            _set.count = 0;
            _set.band = 5.f;
        }

        void update( const openvdb::FloatGrid::ConstPtr&, const openvdb::Vec3fGrid::ConstPtr& ) {}

        void setBoxes( const BoraColliderSet& s ) { _set = s; }

        float signedDistance( const Vec3f& p ) const
        {
            if( _set.count == 0 ) return 5.f;
            float v[3];
            bora_collider_lerp( &_set, (int)_grid.nx(), (int)_grid.ny(), (int)_grid.nz(), p.x, p.y, p.z, BORA_COLLIDER_PHI, v );
            return v[0];
        }

        Vec3f normal( const Vec3f& p ) const
        {
            if( _set.count == 0 ) return Vec3f( 0.f );
            float v[3];
            bora_collider_lerp( &_set, (int)_grid.nx(), (int)_grid.ny(), (int)_grid.nz(), p.x, p.y, p.z, BORA_COLLIDER_NORMAL, v );
            return Vec3f( v[0], v[1], v[2] );
        }

        Vec3f velocity( const Vec3f& p ) const
        {
            if( _set.count == 0 ) return Vec3f( 0.f );
            float v[3];
            bora_collider_lerp( &_set, (int)_grid.nx(), (int)_grid.ny(), (int)_grid.nz(), p.x, p.y, p.z, BORA_COLLIDER_VELOCITY, v );
            return Vec3f( v[0], v[1], v[2] );
        }

        float curvature( const Vec3f& ) const { return 0.f; }
};

BORA_NAMESPACE_END
