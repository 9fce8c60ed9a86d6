// Check of the host-state step's ready lists (ready_lists, host_common.hpp)
// on random meshes: a grid of quads numbered in a scrambled order with
// random boundary gaps, for several element counts and chunk counts. Every
// element, interior edge and boundary face is listed exactly once; each
// element's chunk is at least its own and its face neighbours', each edge's
// at least both its elements', each boundary face's its element's; every
// list is in index order within its chunk. Host build; prints one line,
// exits 1 on failure.
#include <algorithm>
#include <cstdio>
#include <numeric>
#include <random>

#include "host_common.hpp"

using namespace dgswe;

static int failures = 0;
static void expect(bool ok, const char* what, long a, long b) {
    if (!ok && failures++ < 10) std::printf("FAIL %s (%ld, %ld)\n", what, a, b);
}

int main() {
    std::mt19937_64 rng(7);
    long cases = 0;
    for (int nx : {1, 2, 3, 7, 40}) {
        for (int ny : {1, 3, 25}) {
            for (int chunks : {1, 8, 16}) {
                const int64_t K = (int64_t)nx * ny;
                // a scrambled numbering of the grid's cells
                std::vector<int64_t> id(K);
                std::iota(id.begin(), id.end(), 0);
                std::shuffle(id.begin(), id.end(), rng);
                auto at = [&](int i, int j) { return id[(int64_t)j * nx + i]; };
                std::vector<std::array<int64_t, 4>> nb(K, {-1, -1, -1, -1});
                std::vector<int64_t> left, right, bface;
                std::bernoulli_distribution cut(0.1);  // an interior face left as a boundary
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i) {
                        const int64_t k = at(i, j);
                        // faces 0 south, 1 east, 2 north, 3 west
                        if (i + 1 < nx && !cut(rng)) {
                            const int64_t r = at(i + 1, j);
                            nb[k][1] = r;
                            nb[r][3] = k;
                            left.push_back(k * 4 + 1);
                            right.push_back(r * 4 + 3);
                        } else {
                            bface.push_back(k * 4 + 1);
                            if (i + 1 < nx) bface.push_back(at(i + 1, j) * 4 + 3);
                        }
                        if (j + 1 < ny) {
                            const int64_t u = at(i, j + 1);
                            nb[k][2] = u;
                            nb[u][0] = k;
                            left.push_back(k * 4 + 2);
                            right.push_back(u * 4 + 0);
                        } else {
                            bface.push_back(k * 4 + 2);
                        }
                        if (j == 0) bface.push_back(k * 4 + 0);
                        if (i == 0) bface.push_back(k * 4 + 3);
                    }
                const ReadyLists r = ready_lists(K, chunks, nb, left, right, bface);
                const int64_t per = std::max<int64_t>(1, (K + chunks - 1) / chunks);
                auto chunk = [&](int64_t k) { return (int)(k / per); };
                auto check = [&](const std::vector<int32_t>& list, const std::vector<int64_t>& off,
                                 size_t n, auto need, const char* what) {
                    expect((int)off.size() == chunks + 1 && off[0] == 0 && off[chunks] == (int64_t)n,
                           what, (long)off.size(), (long)n);
                    std::vector<int> seen(n, 0);
                    for (int c = 0; c < chunks; ++c)
                        for (int64_t q = off[c]; q < off[c + 1]; ++q) {
                            const int32_t x = list[q];
                            expect(x >= 0 && (size_t)x < n, what, x, c);
                            if (x < 0 || (size_t)x >= n) continue;
                            seen[x] += 1;
                            expect(need(x) == c, what, x, c);
                            if (q > off[c]) expect(list[q - 1] < x, what, list[q - 1], x);
                        }
                    for (size_t x = 0; x < n; ++x) expect(seen[x] == 1, what, (long)x, seen[x]);
                };
                check(r.elems, r.elem_off, (size_t)K, [&](int64_t k) {
                    int c = chunk(k);
                    for (int f = 0; f < 4; ++f)
                        if (nb[k][f] >= 0) c = std::max(c, chunk(nb[k][f]));
                    return c;
                }, "element");
                check(r.edges, r.edge_off, left.size(), [&](int64_t e) {
                    return std::max(chunk(left[e] >> 2), chunk(right[e] >> 2));
                }, "edge");
                check(r.bfaces, r.bface_off, bface.size(),
                      [&](int64_t b) { return chunk(bface[b] >> 2); }, "boundary face");
                cases += 1;
            }
        }
    }
    if (failures) {
        std::printf("%d failures\n", failures);
        return 1;
    }
    std::printf("ok %ld meshes\n", cases);
    return 0;
}
