// Builds the host kd tree (idwarp_gb300/csrc/idw_host.cpp) of the points in
// argv[1] (raw float64, 3 per point, already merged and lexsorted) with bucket
// size argv[2], and writes to argv[3]: the node count (int32), then per node
// l, u, escape, isLeaf (int32 each), then X (3 float64) and 1/radius
// (float64) per node.  Test driver of tests/test_tree_host.py.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "idw_host.hpp"

int main(int argc, char **argv) {
    if (argc != 4) return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    std::vector<double> p;
    double buf[3];
    while (std::fread(buf, sizeof(double), 3, f) == 3) p.insert(p.end(), buf, buf + 3);
    std::fclose(f);
    idw::FlatTree t;
    idw::build_kdtree(p.data(), int(p.size() / 3), std::atoi(argv[2]), t);
    const int nn = t.nodes();
    FILE *o = std::fopen(argv[3], "wb");
    if (!o) return 4;
    std::fwrite(&nn, sizeof(int), 1, o);
    for (const std::vector<int32_t> *a : {&t.l, &t.u, &t.escape, &t.leaf}) std::fwrite(a->data(), sizeof(int32_t), nn, o);
    std::fwrite(t.X.data(), sizeof(double), 3 * size_t(nn), o);
    std::fwrite(t.oradius.data(), sizeof(double), nn, o);
    std::fclose(o);
    return 0;
}
