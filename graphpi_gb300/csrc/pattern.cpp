// Pattern and MotifGenerator (host).  Behaviour follows the reference's
// src/pattern.cpp:9-245 and src/motif_generator.cpp:5-43.
#include "graphpi/motif_generator.h"
#include "graphpi/pattern.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <stdexcept>

Pattern::Pattern(int size, bool clique) : size_(size), adj_((size_t)size * size, 0) {
    if (clique)
        for (int i = 0; i < size; ++i)
            for (int j = 0; j < i; ++j) add_edge(i, j);
}

Pattern::Pattern(int size, const char* buffer) : size_(size), adj_((size_t)size * size, 0) {
    for (int i = 0; i < size; ++i)
        for (int j = 0; j < size; ++j)
            if (buffer[INDEX(i, j, size)] == '1') add_edge(i, j);
}

Pattern::Pattern(PatternType type) {
    // edge lists of the built-in patterns (src/pattern.cpp:45-129)
    static const int rect[][2] = {{0, 1}, {0, 2}, {1, 3}, {2, 3}};
    static const int qg3[][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}};
    static const int penta[][2] = {{0, 1}, {0, 2}, {1, 3}, {2, 4}, {3, 4}};
    static const int house[][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 3}, {1, 4}, {2, 4}};
    static const int hour[][2] = {{0, 1}, {0, 2}, {0, 4}, {1, 2}, {1, 5}, {2, 3}, {3, 4}, {3, 5}, {4, 5}};
    static const int c6t[][2] = {{0, 1}, {0, 2}, {1, 2}, {1, 3}, {1, 4}, {2, 3}, {2, 5}, {0, 4}, {0, 5}};
    const int(*edges)[2] = nullptr;
    int m = 0;
    switch (type) {
        case Rectangle: size_ = 4; edges = rect; m = 4; break;
        case QG3: size_ = 4; edges = qg3; m = 5; break;
        case Pentagon: size_ = 5; edges = penta; m = 5; break;
        case House: size_ = 5; edges = house; m = 6; break;
        case Hourglass: size_ = 6; edges = hour; m = 9; break;
        case Cycle_6_Tri: size_ = 6; edges = c6t; m = 9; break;
        case Clique_7_Minus: size_ = 7; break;
        default: throw std::invalid_argument("invalid pattern type");
    }
    adj_.assign((size_t)size_ * size_, 0);
    if (type == Clique_7_Minus) {
        // K7 without the edge (5, 6)
        for (int i = 0; i < size_; ++i)
            for (int j = 0; j < i; ++j)
                if (!(i == size_ - 1 && j == size_ - 2)) add_edge(j, i);
        return;
    }
    for (int e = 0; e < m; ++e) add_edge(edges[e][0], edges[e][1]);
}

Pattern::Pattern(const Pattern& p) : size_(p.size_), adj_(p.adj_) {}

Pattern::~Pattern() {}

void Pattern::add_edge(int x, int y) {
    adj_[INDEX(x, y, size_)] = 1;
    adj_[INDEX(y, x, size_)] = 1;
}

void Pattern::del_edge(int x, int y) {
    adj_[INDEX(x, y, size_)] = 0;
    adj_[INDEX(y, x, size_)] = 0;
}

bool Pattern::check_connected() const {
    if (size_ == 0) return true;
    std::vector<char> seen(size_, 0);
    std::vector<int> stack{0};
    seen[0] = 1;
    int reached = 1;
    while (!stack.empty()) {
        int x = stack.back();
        stack.pop_back();
        for (int y = 0; y < size_; ++y)
            if (adj_[INDEX(x, y, size_)] && !seen[y]) {
                seen[y] = 1;
                ++reached;
                stack.push_back(y);
            }
    }
    return reached == size_;
}

void Pattern::count_all_isomorphism(std::set<std::set<int> >& s) const {
    std::vector<int> perm(size_);
    std::iota(perm.begin(), perm.end(), 0);
    do {
        std::set<int> key;
        for (int i = 0; i < size_; ++i)
            for (int j = i + 1; j < size_; ++j)
                if (adj_[INDEX(i, j, size_)]) {
                    int a = std::min(perm[i], perm[j]), b = std::max(perm[i], perm[j]);
                    key.insert(a * size_ + b);
                }
        s.insert(key);
    } while (std::next_permutation(perm.begin(), perm.end()));
}

void Pattern::print() const {
    for (int i = 0; i < size_; ++i)
        for (int j = 0; j < size_; ++j)
            if (adj_[INDEX(i, j, size_)]) printf("(%d,%d) ", i, j);
    printf("\n");
}

bool Pattern::is_dag() const {
    // Kahn's algorithm over the directed entries of the matrix.
    std::vector<int> indeg(size_, 0), queue;
    for (int i = 0; i < size_; ++i)
        for (int j = 0; j < size_; ++j)
            if (adj_[INDEX(i, j, size_)] > 0) ++indeg[j];
    for (int i = 0; i < size_; ++i)
        if (indeg[i] == 0) queue.push_back(i);
    for (size_t h = 0; h < queue.size(); ++h) {
        int x = queue[h];
        for (int j = 0; j < size_; ++j)
            if (adj_[INDEX(x, j, size_)] > 0 && --indeg[j] == 0) queue.push_back(j);
    }
    return (int)queue.size() == size_;
}

// ---------------------------------------------------------------------------
// MotifGenerator: walk the upper-triangle pairs (0,1),(0,2)..(n-2,n-1),
// trying "edge present" before "edge absent"; keep a pattern when it is
// connected and no relabelling of it was kept before.

void MotifGenerator::extend(std::vector<Pattern>& out, std::set<int>& edges, Pattern& p, int i, int j) {
    if (i == size - 1) {
        if (!seen.count(edges) && p.check_connected()) {
            out.push_back(p);
            p.count_all_isomorphism(seen);
        }
        return;
    }
    int ni = (j == size - 1) ? i + 1 : i;
    int nj = (j == size - 1) ? i + 2 : j + 1;
    edges.insert(i * size + j);
    p.add_edge(i, j);
    extend(out, edges, p, ni, nj);
    p.del_edge(i, j);
    edges.erase(i * size + j);
    extend(out, edges, p, ni, nj);
}

std::vector<Pattern> MotifGenerator::generate() {
    seen.clear();
    std::vector<Pattern> out;
    if (size < 1) return out;
    std::set<int> edges;
    Pattern p(size);
    extend(out, edges, p, 0, 1);
    return out;
}
