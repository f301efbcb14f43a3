// BTEMesh.h -- mesh container of the StaticBTESolver API.
//
// Public members and constructors as in the reference's
// includes/StaticBTESolver/BTEMesh.h:18-44: a COMSOL .mphtxt reader scaled by
// L_x/L_y/L_z (src/BTEMesh.cpp:7-130) and the uniform 1D mesh generator
// (src/BTEMesh.cpp:132-147).
#ifndef STATICBTESOLVER_GB300_BTEMESH_H
#define STATICBTESOLVER_GB300_BTEMESH_H

#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "utility.h"

class BTEMesh {
public:
    int dim{};
    double L_x{}, L_y{}, L_z{};
    std::vector<std::shared_ptr<staticbtesolver::Point>> meshPts;
    std::vector<std::shared_ptr<staticbtesolver::Segment>> elements1D;
    std::vector<std::shared_ptr<staticbtesolver::Triangle>> elements2D;
    std::vector<std::shared_ptr<staticbtesolver::Tetrahedron>> elements3D;

    BTEMesh() = default;
    // 2D/3D mesh from an opened COMSOL .mphtxt stream; coordinates are scaled by L_x/L_y/L_z.
    BTEMesh(std::ifstream& inFile, double L_x, double L_y = 0, double L_z = 0);
    // Uniform 1D mesh of N_cell cells over [0, L_x].
    BTEMesh(int N_cell, double L_x);
    BTEMesh(const BTEMesh&) = delete;
};

#endif
