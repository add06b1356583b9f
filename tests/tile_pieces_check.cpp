// Checks the tile-piece planner of the FP32 step (meso_host::tile_pieces / split_ngroup) over a grid
// of tile counts, chunk counts and run counts: every chunk of every tile in exactly one piece, each
// (tile, group) at most once with group < ngroup, runs < split, and the runs' chunk totals within
// one run length of each other.  Prints "ok" or the first failing shape.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "host/fp32_host.h"

int main() {
    const int nts[] = {1, 2, 5, 6, 22, 137, 151, 152, 153, 162, 304, 341, 1000};
    const int chs[] = {1, 2, 3, 13, 27, 160, 161};
    const int sps[] = {1, 7, 148, 152};
    for (int nt : nts)
        for (int ch : chs)
            for (int sp : sps) {
                const int ng = meso_host::split_ngroup(nt, ch, sp);
                const auto ps = meso_host::tile_pieces(nt, ch, ng, sp);
                std::vector<int> seen((size_t)nt * ng, 0), cover((size_t)nt * ch, 0);
                std::vector<long> load(sp, 0);
                for (const auto &p : ps) {
                    if (p.tile < 0 || p.tile >= nt || p.grp < 0 || p.grp >= ng || p.run < 0 || p.run >= sp ||
                        p.ch0 < 0 || p.ch1 > ch || p.ch0 >= p.ch1) {
                        std::printf("bad piece: tiles %d chunks %d runs %d\n", nt, ch, sp);
                        return 1;
                    }
                    seen[(size_t)p.tile * ng + p.grp]++;
                    for (int c = p.ch0; c < p.ch1; ++c) cover[(size_t)p.tile * ch + c]++;
                    load[p.run] += p.ch1 - p.ch0;
                }
                if (*std::max_element(seen.begin(), seen.end()) > 1 ||
                    *std::min_element(cover.begin(), cover.end()) != 1 ||
                    *std::max_element(cover.begin(), cover.end()) != 1) {
                    std::printf("not a partition: tiles %d chunks %d runs %d\n", nt, ch, sp);
                    return 1;
                }
                const long total = (long)nt * ch, ideal = (total + sp - 1) / sp;
                if (*std::max_element(load.begin(), load.end()) > ideal + std::max(ch, 2)) {
                    std::printf("unbalanced: tiles %d chunks %d runs %d\n", nt, ch, sp);
                    return 1;
                }
            }
    // equal groups per tile (split 0)
    for (int nt : nts)
        for (int ch : chs)
            for (int ng = 1; ng <= std::min(ch, 8); ++ng) {
                const auto ps = meso_host::tile_pieces(nt, ch, ng, 0);
                std::vector<int> cover((size_t)nt * ch, 0);
                for (const auto &p : ps)
                    for (int c = p.ch0; c < p.ch1; ++c) cover[(size_t)p.tile * ch + c]++;
                if (*std::min_element(cover.begin(), cover.end()) != 1 ||
                    *std::max_element(cover.begin(), cover.end()) != 1) {
                    std::printf("groups not a partition: tiles %d chunks %d groups %d\n", nt, ch, ng);
                    return 1;
                }
            }
    std::printf("ok\n");
    return 0;
}
