// DataLoader — text edge lists, the raw binary CSR format, and complete
// graphs into a Graph.  Same interface as the reference's DataLoader
// (include/dataloader.h:28-48 of thu-pacman/GraphPi).
#pragma once
#include <map>
#include <utility>
#include <vector>
#include "graph.h"

enum DataType { Patents, Orkut, complete8, LiveJournal, MiCo, Twitter, CiteSeer, Wiki_Vote, Invalid };

// Triangle counts of the classic datasets (include/dataloader.h:19-25).
const long long Patents_tri_cnt = 7515023LL;
const long long LiveJournal_tri_cnt = 177820130LL;
const long long MiCo_tri_cnt = 12534960LL;
const long long CiteSeer_tri_cnt = 1166LL;
const long long Wiki_Vote_tri_cnt = 608389LL;
const long long Orkut_tri_cnt = 627584181LL;
const long long Twitter_tri_cnt = 34824916864LL;

class DataLoader {
public:
    // oriented_type 0: keep ids, 1: high degree first, 2: low degree first.
    // For a DataType without a known triangle count, tri_cnt is computed on
    // the GPU.
    bool load_data(Graph*& g, DataType type, const char* path, int oriented_type = 0);
    bool load_complete(Graph*& g, int clique_size);

private:
    bool general_load_data(Graph*& g, DataType type, const char* path, int oriented_type);
    bool twitter_load_data(Graph*& g, DataType type, const char* path, int oriented_type);
    // CSR of both-direction pairs built on the GPU; false without a device
    static bool gpu_build_csr(Graph* g, const std::vector<std::pair<int, int> >& e);
    std::map<int, int> id;
};
