// Host-side air-mesh generator for the bijectivity scaffold (oc_airmesh.cpp).
#pragma once

#include "optcuts_gpu.h"

#include <string>
#include <vector>

namespace oc {

struct AirMesh {
    std::vector<double> V;   // nAirV x 2: boundary vertices (loop by loop), box points, Steiner points
    std::vector<int> F;      // nAirF x 3, counter-clockwise
    std::vector<int> bnd;    // air vertex i < nBnd is mesh vertex bnd[i]
    int nBnd = 0;
};

// Air mesh for the UV layout (UV nV x 2, F nF x 3) with box margin and
// segment length from avgEdgeLen (the mesh's rest average edge length);
// minAngleDeg > 0 refines the air region towards that minimum angle.
constexpr double kAirMinAngle = 20.0;   // Triangle's "q" default
int air_mesh_build(const double* UV, int nV, const int* F, int nF, double avgEdgeLen, AirMesh& out,
                   std::string* err, double minAngleDeg = kAirMinAngle);
// the same in two parts: what depends on the topology only -- the boundary
// loops of F (bnd loop by loop, loop l = bnd[loopStart[l] .. loopStart[l +
// 1])) and the first triangle of each connected component (seedTris, 3
// vertex ids each) -- and the air mesh for a UV layout from those
int air_mesh_boundary(int nV, const int* F, int nF, std::vector<int>& bnd, std::vector<int>& loopStart,
                      std::vector<int>& seedTris, std::string* err);
int air_mesh_build_loops(const double* UV, int nV, const std::vector<int>& bnd, const std::vector<int>& loopStart,
                         const std::vector<int>& seedTris, double avgEdgeLen, AirMesh& out, std::string* err,
                         double minAngleDeg = kAirMinAngle);

} // namespace oc
