// Loads a graph through the C++ DataLoader (reference API,
// include/dataloader.h:28-48) and prints its CSR, so tests can compare the
// loaders.  usage: load_dump DATASET PATH ORIENTED_TYPE
// Output: "v e max_degree tri", then vertex[0..v], then edge[0..e).
#include <cstdio>
#include <cstdlib>

#include "graphpi/common.h"
#include "graphpi/dataloader.h"
#include "graphpi/graph.h"

int main(int argc, char* argv[]) {
    if (argc < 4) return 2;
    Graph* g = nullptr;
    DataLoader D;
    DataType type;
    GetDataType(type, argv[1]);
    if (type == DataType::Invalid || !D.load_data(g, type, argv[2], atoi(argv[3]))) {
        printf("load failed\n");
        return 1;
    }
    printf("%d %u %d %lld\n", g->v_cnt, g->e_cnt, g->max_degree, g->tri_cnt);
    for (int i = 0; i <= g->v_cnt; ++i) printf("%u ", g->vertex[i]);
    printf("\n");
    for (unsigned i = 0; i < g->e_cnt; ++i) printf("%d ", g->edge[i]);
    printf("\n");
    delete g;
    return 0;
}
