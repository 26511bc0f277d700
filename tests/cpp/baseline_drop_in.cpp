// A GraphPi driver written against the reference's C++ API
// (tianhe/baseline_test.cpp of thu-pacman/GraphPi): only the include paths
// and the link line differ.  usage: baseline_drop_in DATASET PATH SIZE ADJ
#include <cassert>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "graphpi/common.h"
#include "graphpi/dataloader.h"
#include "graphpi/graph.h"
#include "graphpi/pattern.h"
#include "graphpi/schedule.h"

int main(int argc, char* argv[]) {
    if (argc < 5) {
        printf("Usage: %s dataset_name graph_file pattern_size pattern_adjacency_matrix\n", argv[0]);
        return 2;
    }
    Graph* g;
    DataLoader D;
    DataType type;
    GetDataType(type, argv[1]);
    if (type == DataType::Invalid || !D.load_data(g, type, argv[2])) {
        printf("load failed\n");
        return 1;
    }
    Pattern p(atoi(argv[3]), argv[4]);
    bool valid;
    Schedule schedule(p, valid, 1, 1, true, g->v_cnt, g->e_cnt, g->tri_cnt);
    assert(valid);
    double t1 = get_wall_time();
    long long ans = g->pattern_matching(schedule, 24);
    double t2 = get_wall_time();
    printf("ans %lld\n", ans);
    printf("tri %lld\n", g->tri_cnt);
    printf("time %.6lf\n", t2 - t1);
    delete g;
    return 0;
}
