// Graph — the data graph as a symmetric CSR, plus the GPU entry points.
// Same public fields and methods as the reference's Graph
// (include/graph.h:7-61 of thu-pacman/GraphPi): `edge`/`vertex` hold the
// host CSR; the first counting call uploads it to HBM (relabelled by degree)
// and later calls reuse the device copy until the Graph is destroyed.
// thread_count is accepted for source compatibility and ignored: work runs
// on the current CUDA device.
#pragma once
#include <cstdint>
#include "../gpm.h"
#include "schedule.h"

class Graph {
public:
    int v_cnt;            // number of vertices
    unsigned int e_cnt;   // number of directed edges (2x undirected)
    long long tri_cnt;    // number of triangles (-1: unknown, computed on demand)
    double max_running_time = 60 * 60 * 24;  // seconds (kept for API parity)

    int* edge;              // neighbours, sorted per vertex
    unsigned int* vertex;   // v's neighbours are edge[vertex[v] .. vertex[v+1])
    int max_degree;

    Graph();
    ~Graph();
    Graph(const Graph&) = delete;
    Graph& operator=(const Graph&) = delete;

    int intersection_size(int v1, int v2);
    int intersection_size_clique(int v1, int v2);

    long long triangle_counting();
    long long triangle_counting_mt(int thread_count);

    // Returns the count when it fits in a signed 64-bit integer; otherwise
    // prints a message to stderr and returns -1 (use pattern_matching_u128).
    long long pattern_matching(const Schedule& schedule, int thread_count, bool clique = false);
    long long pattern_matching_mpi(const Schedule& schedule, int thread_count, bool clique = false);
    gpm_u128 pattern_matching_u128(const Schedule& schedule);

    // Drops the device copy (next call re-uploads); call after editing the
    // host CSR in place.
    void invalidate_device();
    gpm_graph* device_graph();

private:
    friend class DataLoader;  // hands over the device CSR it built
    gpm_graph* dev_ = nullptr;
};
