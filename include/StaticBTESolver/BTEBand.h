// BTEBand.h -- phonon band list of the StaticBTESolver API
// (reference: includes/StaticBTESolver/BTEBand.h:17-56, src/BTEBand.cpp:8-49).
// One band per line: "GROUP_VELOCITY RELAXATION_TIME Ctot Lr"; reading stops
// at the first line of length <= 1.
#ifndef STATICBTESOLVER_GB300_BTEBAND_H
#define STATICBTESOLVER_GB300_BTEBAND_H

#include <fstream>
#include <iostream>
#include <vector>

#include "utility.h"

using namespace staticbtesolver;

class BTEBand {
    using BandList = std::vector<Band>;
    BandList bands;

public:
    BTEBand() = default;
    explicit BTEBand(std::ifstream& inFile);
    BTEBand(const BTEBand&) = default;
    BTEBand& operator=(const BTEBand&) = default;
    using iterator = BandList::iterator;
    using const_iterator = BandList::const_iterator;
    const_iterator begin() const { return bands.begin(); }
    const_iterator end() const { return bands.end(); }
    std::size_t size() { return bands.size(); }
    std::size_t size() const { return bands.size(); }
    const Band& operator[](std::size_t i) const { return bands[i]; }
    // Additive: append a band (the reference only reads files).
    void push_back(const Band& b) { bands.push_back(b); }
    friend std::ostream& operator<<(std::ostream& os, const BTEBand& band);
};

#endif
