// Graph, DataLoader and common helpers: the reference's C++ API on top of
// the C ABI.  Graph keeps the host CSR in the reference's public fields
// (include/graph.h:9-16) and owns one device copy, created on the first
// GPU call.  Counting always runs on the GPU; without one it throws.
#include <sys/time.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "graphpi/common.h"
#include "graphpi/dataloader.h"
#include "graphpi/graph.h"

namespace {

void check(int rc, const char* what) {
    if (rc != GPM_OK) throw std::runtime_error(std::string(what) + ": " + gpm_last_error());
}

}  // namespace

Graph::Graph() : v_cnt(0), e_cnt(0), tri_cnt(-1), edge(nullptr), vertex(nullptr), max_degree(0) {}

Graph::~Graph() {
    if (dev_) gpm_graph_destroy(dev_);
    delete[] edge;
    delete[] vertex;
}

void Graph::invalidate_device() {
    if (dev_) gpm_graph_destroy(dev_);
    dev_ = nullptr;
}

gpm_graph* Graph::device_graph() {
    if (!dev_) check(gpm_graph_create(v_cnt, vertex, edge, 1, &dev_), "Graph: upload to GPU");
    return dev_;
}

int Graph::intersection_size(int v1, int v2) {
    unsigned a = vertex[v1], b = vertex[v1 + 1], c = vertex[v2], d = vertex[v2 + 1];
    int n = 0;
    while (a < b && c < d) {
        if (edge[a] < edge[c]) ++a;
        else if (edge[c] < edge[a]) ++c;
        else ++n, ++a, ++c;
    }
    return n;
}

int Graph::intersection_size_clique(int v1, int v2) {
    // common neighbours below v2
    unsigned a = vertex[v1], b = vertex[v1 + 1], c = vertex[v2], d = vertex[v2 + 1];
    int n = 0;
    while (a < b && c < d && edge[a] < v2 && edge[c] < v2) {
        if (edge[a] < edge[c]) ++a;
        else if (edge[c] < edge[a]) ++c;
        else ++n, ++a, ++c;
    }
    return n;
}

long long Graph::triangle_counting() { return triangle_counting_mt(1); }

long long Graph::triangle_counting_mt(int) {
    uint64_t t = 0;
    check(gpm_tri_count(device_graph(), &t), "Graph::triangle_counting");
    return (long long)t;
}

gpm_u128 Graph::pattern_matching_u128(const Schedule& schedule) {
    std::vector<int64_t> t = schedule.pack();
    gpm_plan* p = nullptr;
    check(gpm_plan_create(t.data(), (int32_t)t.size(), &p), "Graph::pattern_matching: plan");
    gpm_u128 out{0, 0};
    int rc = gpm_count(device_graph(), p, &out);
    std::string msg = rc ? gpm_last_error() : "";
    gpm_plan_destroy(p);
    if (rc) throw std::runtime_error("Graph::pattern_matching: " + msg);
    return out;
}

long long Graph::pattern_matching(const Schedule& schedule, int, bool clique) {
    gpm_u128 c{0, 0};
    const int n = schedule.get_size();
    const int* adj = schedule.get_adj_mat_ptr();
    bool complete = clique && n >= 3;
    for (int i = 0; i < n && complete; ++i)
        for (int j = 0; j < n; ++j)
            if (i != j && !adj[i * n + j]) complete = false;
    if (complete)  // the clique fast path: same count, no restriction checks
        check(gpm_clique_count(device_graph(), n, &c), "Graph::pattern_matching (clique)");
    else
        c = pattern_matching_u128(schedule);
    if (c.hi != 0 || c.lo > (uint64_t)LLONG_MAX) {
        fprintf(stderr, "Graph::pattern_matching: count exceeds 2^63-1; use pattern_matching_u128\n");
        return -1;
    }
    return (long long)c.lo;
}

long long Graph::pattern_matching_mpi(const Schedule& schedule, int thread_count, bool clique) {
    return pattern_matching(schedule, thread_count, clique);
}

// ---------------------------------------------------------------------------
// DataLoader (src/dataloader.cpp:8-262)

namespace {

// Builds the CSR from directed pairs on the host: sort, dedupe, offsets.
void fill_csr(Graph* g, std::vector<std::pair<int, int> >& e) {
    std::sort(e.begin(), e.end());
    e.erase(std::unique(e.begin(), e.end()), e.end());
    g->e_cnt = (unsigned)e.size();
    g->edge = new int[std::max<size_t>(e.size(), 1)];
    g->vertex = new unsigned[(size_t)g->v_cnt + 1];
    size_t k = 0;
    for (int v = 0; v < g->v_cnt; ++v) {
        g->vertex[v] = (unsigned)k;
        while (k < e.size() && e[k].first == v) {
            g->edge[k] = e[k].second;
            ++k;
        }
    }
    g->vertex[g->v_cnt] = (unsigned)k;
    int md = 0;
    for (int v = 0; v < g->v_cnt; ++v) md = std::max(md, (int)(g->vertex[v + 1] - g->vertex[v]));
    g->max_degree = md;
}

long long table_tri_cnt(DataType t) {
    switch (t) {
        case Patents: return Patents_tri_cnt;
        case LiveJournal: return LiveJournal_tri_cnt;
        case MiCo: return MiCo_tri_cnt;
        case CiteSeer: return CiteSeer_tri_cnt;
        case Wiki_Vote: return Wiki_Vote_tri_cnt;
        case Orkut: return Orkut_tri_cnt;
        case Twitter: return Twitter_tri_cnt;
        default: return -1;
    }
}

// reads all whitespace-separated integers of a text file
bool read_ints(const char* path, std::vector<long long>& out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    std::vector<char> buf(1 << 20);
    long long cur = 0;
    bool in = false, neg = false;
    size_t n;
    while ((n = fread(buf.data(), 1, buf.size(), f)) > 0) {
        for (size_t i = 0; i < n; ++i) {
            char ch = buf[i];
            if (ch >= '0' && ch <= '9') {
                cur = cur * 10 + (ch - '0');
                in = true;
            } else {
                if (in) out.push_back(neg ? -cur : cur);
                in = false;
                cur = 0;
                neg = (ch == '-');
            }
        }
    }
    if (in) out.push_back(neg ? -cur : cur);
    fclose(f);
    return true;
}

void fill_tri_cnt(Graph* g, DataType type) {
    g->tri_cnt = table_tri_cnt(type);
    if (g->tri_cnt >= 0) return;
    try {
        g->tri_cnt = g->triangle_counting_mt(0);
    } catch (const std::exception& ex) {
        fprintf(stderr, "DataLoader: triangle count unavailable (%s); tri_cnt = -1\n", ex.what());
        g->tri_cnt = -1;
    }
}

}  // namespace

// Builds the CSR on the GPU (gpm_graph_from_edges: symmetrise, sort,
// deduplicate, offsets on the device; relabelled by degree like every
// device copy), downloads it in the file's ids into the reference's host
// fields and keeps the device copy for the counting calls.  Returns
// false, with nothing changed, when no CUDA device is present; the host
// builder then does the same steps.
bool DataLoader::gpu_build_csr(Graph* g, const std::vector<std::pair<int, int> >& e) {
    std::vector<int32_t> src, dst;
    src.reserve(e.size() / 2);
    dst.reserve(e.size() / 2);
    for (const auto& p : e)
        if (p.first < p.second) {  // both directions are in e; one is enough
            src.push_back(p.first);
            dst.push_back(p.second);
        }
    gpm_graph* dev = nullptr;
    const int rc = gpm_graph_from_edges(g->v_cnt, (int64_t)src.size(), src.data(), dst.data(), 1, &dev);
    if (rc == GPM_ERR_NO_DEVICE) return false;
    check(rc, "DataLoader: GPU CSR build");
    int64_t ecnt = 0, md = 0;
    check(gpm_graph_stats(dev, nullptr, &ecnt, &md, nullptr), "DataLoader: GPU CSR build");
    g->e_cnt = (unsigned)ecnt;
    g->edge = new int[std::max<int64_t>(ecnt, 1)];
    g->vertex = new unsigned[(size_t)g->v_cnt + 1];
    check(gpm_graph_download(dev, g->vertex, g->edge), "DataLoader: GPU CSR download");
    g->max_degree = (int)md;
    g->dev_ = dev;
    return true;
}

bool DataLoader::load_data(Graph*& g, DataType type, const char* path, int oriented_type) {
    if (type == Twitter) return twitter_load_data(g, type, path, oriented_type);
    if (type == Invalid) {
        printf("invalid DataType!\n");
        return false;
    }
    return general_load_data(g, type, path, oriented_type);
}

bool DataLoader::general_load_data(Graph*& g, DataType type, const char* path, int oriented_type) {
    std::vector<long long> ints;
    if (!read_ints(path, ints)) {
        printf("File not found. %s\n", path);
        return false;
    }
    if (ints.size() < 2) return false;
    g = new Graph();
    g->v_cnt = (int)ints[0];
    long long expect_e = ints[1] * 2;
    std::vector<std::pair<int, int> > e;
    e.reserve((ints.size() - 2));
    id.clear();
    int next_id = 0;
    std::vector<int> degree;
    for (size_t i = 2; i + 1 < ints.size(); i += 2) {
        int x = (int)ints[i], y = (int)ints[i + 1];
        if (x == y) {  // self loops are dropped (src/dataloader.cpp:73-78)
            expect_e -= 2;
            continue;
        }
        auto ix = id.find(x);
        if (ix == id.end()) ix = id.emplace(x, next_id++).first;
        auto iy = id.find(y);
        if (iy == id.end()) iy = id.emplace(y, next_id++).first;
        x = ix->second;
        y = iy->second;
        e.push_back(std::make_pair(x, y));
        e.push_back(std::make_pair(y, x));
    }
    if (next_id != g->v_cnt || (long long)e.size() != expect_e) {
        if (next_id != g->v_cnt) printf("vertex number error!\n");
        if ((long long)e.size() != expect_e) printf("edge number error!\n");
        delete g;
        g = nullptr;
        return false;
    }
    if (oriented_type != 0) {
        degree.assign(g->v_cnt, 0);
        for (auto& p : e) ++degree[p.first];
        std::vector<int> order(g->v_cnt), new_id(g->v_cnt);
        for (int i = 0; i < g->v_cnt; ++i) order[i] = i;
        if (oriented_type == 1)
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return degree[a] > degree[b]; });
        else
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return degree[a] < degree[b]; });
        for (int i = 0; i < g->v_cnt; ++i) new_id[order[i]] = i;
        for (auto& p : e) p = std::make_pair(new_id[p.first], new_id[p.second]);
    }
    if (!gpu_build_csr(g, e)) fill_csr(g, e);
    printf("Success! There are %d nodes and %u edges.\n", g->v_cnt, g->e_cnt);
    fflush(stdout);
    fill_tri_cnt(g, type);
    return true;
}

bool DataLoader::twitter_load_data(Graph*& g, DataType type, const char* path, int) {
    // raw little-endian uint32: v_cnt, e_cnt, max_degree, vertex[v_cnt+1], edge[e_cnt]
    FILE* f = fopen(path, "rb");
    if (!f) {
        printf("File not found. %s\n", path);
        return false;
    }
    unsigned hdr[3];
    if (fread(hdr, sizeof(unsigned), 3, f) != 3) {
        fclose(f);
        return false;
    }
    g = new Graph();
    g->v_cnt = (int)hdr[0];
    g->e_cnt = hdr[1];
    g->max_degree = (int)hdr[2];
    g->vertex = new unsigned[(size_t)g->v_cnt + 1];
    g->edge = new int[std::max<size_t>(g->e_cnt, 1)];
    bool ok = fread(g->vertex, sizeof(unsigned), (size_t)g->v_cnt + 1, f) == (size_t)g->v_cnt + 1 &&
              fread(g->edge, sizeof(int), g->e_cnt, f) == g->e_cnt && g->vertex[0] == 0 &&
              g->vertex[g->v_cnt] == g->e_cnt;
    fclose(f);
    if (!ok) {
        printf("malformed binary graph %s\n", path);
        delete g;
        g = nullptr;
        return false;
    }
    fill_tri_cnt(g, type);
    return true;
}

bool DataLoader::load_complete(Graph*& g, int clique_size) {
    if (clique_size < 2) return false;
    g = new Graph();
    g->v_cnt = clique_size;
    std::vector<std::pair<int, int> > e;
    for (int i = 0; i < clique_size; ++i)
        for (int j = 0; j < clique_size; ++j)
            if (i != j) e.push_back(std::make_pair(i, j));
    fill_csr(g, e);
    // K_n has C(n, 3) triangles
    g->tri_cnt = (long long)clique_size * (clique_size - 1) * (clique_size - 2) / 6;
    return true;
}

// ---------------------------------------------------------------------------
// common.h

double get_wall_time() {
    struct timeval t;
    if (gettimeofday(&t, nullptr)) return 0;
    return (double)t.tv_sec + (double)t.tv_usec * 1e-6;
}

void PatternType_printer(PatternType type) {
    static const char* names[] = {"Rectangle", "QG3", "Pentagon", "House", "Hourglass", "Cycle_6_Tri", "Clique_7_Minus"};
    if (type >= Rectangle && type <= Clique_7_Minus) printf("%s\n", names[type]);
}

bool is_equal_adj_mat(const int* a, const int* b, int size) {
    return std::equal(a, a + size * size, b);
}

void GetDataType(DataType& type, const std::string str) {
    static const std::pair<const char*, DataType> names[] = {
        {"Patents", Patents}, {"Orkut", Orkut}, {"complete8", complete8}, {"LiveJournal", LiveJournal},
        {"MiCo", MiCo},       {"Twitter", Twitter}, {"CiteSeer", CiteSeer}, {"Wiki-Vote", Wiki_Vote}};
    type = Invalid;
    for (const auto& n : names)
        if (str == n.first) type = n.second;
}
