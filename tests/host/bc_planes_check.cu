// Host check of bc_plane_cells / bc_plane_cell (ia_bc.cuh), the enumeration the velocity BC, the
// periodic pressure ghosts and the VOF ghost fills launch over: every enumerated cell lies in the
// grid, the enumerated set is the union of the planes c[e] in {0, 1, n_e - 1}, and numbers past the
// count are rejected.  Exit status 0 on success.
#include <cstdio>
#include <set>
#include <tuple>

#include "../../interfaceadvection.jl_gb300/csrc/ia_bc.cuh"

using namespace ia;

int main() {
    int bad = 0;
    const int64_t sizes[][3] = {{10, 7, 5}, {128, 64, 6}, {1, 3, 2}, {4, 4, 4}};
    for (int D = 2; D <= 3; ++D)
        for (int per = 0; per < (1 << D); ++per)
            for (const auto& sz : sizes) {
                const int64_t Nint[3] = {sz[0], sz[1], D == 3 ? sz[2] : 1};
                const Grid g = make_grid(D, per, Nint);
                std::set<std::tuple<int, int, int>> got, want;
                const long long n = bc_plane_cells(g);
                for (long long t = 0; t < n + 100; ++t) {
                    int c[3] = {-1, -1, -1};
                    const bool ok = bc_plane_cell(g, t, c);
                    if (ok != (t < n)) ++bad;
                    if (!ok) continue;
                    for (int e = 0; e < 3; ++e)
                        if (c[e] < 0 || c[e] >= g.n[e]) ++bad;
                    got.insert({c[0], c[1], c[2]});
                }
                for (int z = 0; z < g.n[2]; ++z)
                    for (int y = 0; y < g.n[1]; ++y)
                        for (int x = 0; x < g.n[0]; ++x) {
                            const int c[3] = {x, y, z};
                            bool on = false;
                            for (int e = 0; e < D; ++e)
                                if (c[e] == 0 || c[e] == 1 || c[e] == g.n[e] - 1) on = true;
                            if (on) want.insert({x, y, z});
                        }
                if (got != want) {
                    ++bad;
                    std::printf("set mismatch: D=%d per=%d n=%d,%d,%d\n", D, per, g.n[0], g.n[1], g.n[2]);
                }
            }
    std::printf(bad ? "FAIL %d\n" : "ok\n", bad);
    return bad != 0;
}
