// Reverse Cuthill-McKee over the face-neighbour graph of the cells.
#include "renumber.h"

#include <algorithm>
#include <numeric>

namespace meso_host {

Renumbering renumber(const meso_mesh_desc &m, bool identity) {
    Renumbering r;
    const int C = m.ncell, F = m.nface;
    r.cell_new2old.resize(C);
    if (identity) {
        std::iota(r.cell_new2old.begin(), r.cell_new2old.end(), 0);
    } else {
        std::vector<int> deg(C);
        for (int c = 0; c < C; ++c) deg[c] = m.cell_nbr_ptr[c + 1] - m.cell_nbr_ptr[c];
        std::vector<char> seen(C, 0);
        std::vector<int> order;
        order.reserve(C);
        std::vector<int> by_deg(C);
        std::iota(by_deg.begin(), by_deg.end(), 0);
        std::stable_sort(by_deg.begin(), by_deg.end(), [&](int a, int b) { return deg[a] < deg[b]; });
        std::vector<int> nb;
        for (int start : by_deg) {
            if (seen[start]) continue;
            size_t head = order.size();
            order.push_back(start);
            seen[start] = 1;
            while (head < order.size()) {
                int c = order[head++];
                nb.clear();
                for (int j = m.cell_nbr_ptr[c]; j < m.cell_nbr_ptr[c + 1]; ++j) {
                    int n = m.cell_nbr[j];
                    if (!seen[n]) {
                        seen[n] = 1;
                        nb.push_back(n);
                    }
                }
                std::stable_sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
                order.insert(order.end(), nb.begin(), nb.end());
            }
        }
        std::reverse(order.begin(), order.end());
        r.cell_new2old = order;
    }
    r.cell_old2new.assign(C, 0);
    for (int i = 0; i < C; ++i) r.cell_old2new[r.cell_new2old[i]] = i;
    r.face_new2old.resize(F);
    std::iota(r.face_new2old.begin(), r.face_new2old.end(), 0);
    if (!identity) {
        auto key = [&](int f) {
            int a = r.cell_old2new[m.face_cell[2 * f]], b = r.cell_old2new[m.face_cell[2 * f + 1]];
            return std::make_pair(a, b);
        };
        std::stable_sort(r.face_new2old.begin(), r.face_new2old.end(), [&](int x, int y) { return key(x) < key(y); });
    }
    r.face_old2new.assign(F, 0);
    for (int i = 0; i < F; ++i) r.face_old2new[r.face_new2old[i]] = i;
    return r;
}

}  // namespace meso_host
