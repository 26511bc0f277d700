// MotifGenerator — every connected k-vertex pattern up to isomorphism, in the
// reference's generation order (include/motif_generator.h:5-13).
#pragma once
#include <set>
#include <vector>
#include "pattern.h"

class MotifGenerator {
public:
    explicit MotifGenerator(int input_size) : size(input_size) {}
    std::vector<Pattern> generate();

private:
    int size;
    std::set<std::set<int> > seen;
    void extend(std::vector<Pattern>& out, std::set<int>& edges, Pattern& p, int i, int j);
};
