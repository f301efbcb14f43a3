// BTEBoundaryCondition.h -- boundary-condition list of the StaticBTESolver API
// (reference: includes/StaticBTESolver/BTEBoundaryCondition.h:15-55,
// src/BTEBoundaryCondition.cpp:7-47).  File: a count, two skipped lines, then
// "entity type temperature" rows; index is stored as -entity-1.
#ifndef STATICBTESOLVER_GB300_BTEBOUNDARYCONDITION_H
#define STATICBTESOLVER_GB300_BTEBOUNDARYCONDITION_H

#include <fstream>
#include <iostream>
#include <vector>

#include "utility.h"

class BTEBoundaryCondition {
    using BoundaryConditionList = std::vector<staticbtesolver::BoundaryCondition>;

public:
    BoundaryConditionList boundaryConditions;
    BTEBoundaryCondition() = default;
    explicit BTEBoundaryCondition(std::ifstream& inFile);
    BTEBoundaryCondition(const BTEBoundaryCondition&) = default;
    BTEBoundaryCondition& operator=(const BTEBoundaryCondition&) = default;
    using iterator = BoundaryConditionList::iterator;
    using const_iterator = BoundaryConditionList::const_iterator;
    const_iterator begin() const { return boundaryConditions.begin(); }
    const_iterator end() const { return boundaryConditions.end(); }
    std::size_t size() const { return boundaryConditions.size(); }
    const staticbtesolver::BoundaryCondition& operator[](std::size_t i) const { return boundaryConditions[i]; }
    friend std::ostream& operator<<(std::ostream& os, const BTEBoundaryCondition& bc);
};

#endif
