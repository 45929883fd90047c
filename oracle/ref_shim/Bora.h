// Host-only replacement for the reference's umbrella header (base/header/Bora.h).
//
// ORACLE INFRASTRUCTURE. This header lets the reference's own FLIP sources
// (base/source/{SparseFrame,Rasterization,FluidProjection,BLAS,FieldOP,FLIPMethod}.cu
// and {ArrayUtils,LinearSystemSolver,Particles}.cpp) compile unmodified with g++ for
// the host CPU, so that the reference itself can be run as a test oracle and as the
// timed CPU baseline. It is never linked into the product library.
//
// What it provides in place of the reference's Foundation.h (base/header/Foundation.h:58-107):
//   * the C++ standard headers the reference expects, and the BORA_* macros with the
//     CUDA qualifiers removed (base/header/Foundation.h:11-21);
//   * host stand-ins for the handful of CUDA runtime calls used on the path
//     (managed allocation, memcpy/memset, atomicAdd), see cuda_host.h;
//   * LaunchCudaDevice as an OpenMP parallel loop (the reference maps it to
//     thrust::for_each over a counting iterator, base/header/LauncherCuda.h:13-17);
//   * minimal declarations of the glm, OpenGL and OpenVDB names that appear in the
//     headers' signatures, so they parse. Nothing is drawn or sampled through them.
// Only the subset of reference headers that the FLIP path needs is included,
// in the order of the reference's own Bora.h.
#pragma once

#include "shim_foundation.h"

#include <Definitions.h>
#include <TimeWatch.h>
#include <MemoryUtils.h>
#include <MathUtils.h>
#include <Random.h>
#include <Vector2.h>
#include <Vector3.h>
#include <Vector4.h>
#include <Matrix22.h>
#include <Matrix33.h>
#include <Matrix44.h>
#include <Quaternion.h>
#include <AABB2.h>
#include <AABB3.h>
// Grid::draw (base/header/Grid.h:506) names this helper from OpenGLUtils.h; a no-op here.
namespace Bora { inline void DrawCube( const Vec3f&, const Vec3f& ) {} }
#include <Noise.h>
#include <Array.h>
#include <ArrayUtils.h>
#include <Particles.h>
#include <Grid.h>
#include <DenseField.h>
#include <ScalarDenseField.h>
#include <VectorDenseField.h>
#include <MarkerDenseField.h>
#include <IndexDenseField.h>
#include <SparseFrame.h>
#include <SparseField.h>
#include <FieldOP.h>
#include <SparseMatrix.h>
#include <BLAS.h>
#include <LinearSystemSolver.h>
#include <FluidProjection.h>
#include <Rasterization.h>
#include "CollisionSource.h"
#include <FLIPMethod.h>

using namespace Bora;
