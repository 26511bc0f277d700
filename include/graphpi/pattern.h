// Pattern — a small undirected query graph held as a dense adjacency
// matrix.  Same public interface as the reference's Pattern
// (include/pattern.h:20-43 of thu-pacman/GraphPi).
#pragma once
#include <set>
#include <vector>

#ifndef INDEX
#define INDEX(x, y, n) ((x) * (n) + (y))
#endif

// Built-in patterns (include/pattern.h:10-18).
enum PatternType { Rectangle, QG3, Pentagon, House, Hourglass, Cycle_6_Tri, Clique_7_Minus };

class Pattern {
public:
    explicit Pattern(int size, bool clique = false);
    Pattern(int size, const char* buffer);  // row-major '0'/'1' matrix
    Pattern(PatternType type);
    Pattern(const Pattern& p);
    ~Pattern();

    void add_edge(int x, int y);
    void del_edge(int x, int y);
    inline void add_ordered_edge(int x, int y) { adj_[INDEX(x, y, size_)] = 1; }
    inline int get_size() const { return size_; }
    inline const int* get_adj_mat_ptr() const { return adj_.data(); }

    bool check_connected() const;
    // Inserts the edge set of every relabelling of this pattern into s.
    void count_all_isomorphism(std::set<std::set<int> >& s) const;
    void print() const;
    bool is_dag() const;

private:
    Pattern& operator=(const Pattern&);
    int size_;
    std::vector<int> adj_;
};
