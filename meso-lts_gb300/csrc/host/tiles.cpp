// Tile planner for the FP32 step.  See tiles.h.
#include "tiles.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace meso_host {

namespace {

void rcb(const meso_mesh_desc &m, std::vector<int> &ids, size_t lo, size_t hi, int T,
         std::vector<std::pair<size_t, size_t>> &out) {
    const size_t n = hi - lo;
    if (n <= (size_t)T) {
        out.emplace_back(lo, hi);
        return;
    }
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (size_t i = lo; i < hi; ++i)
        for (int k = 0; k < 3; ++k) {
            double v = m.cell_pos[3 * (size_t)ids[i] + k];
            mn[k] = std::min(mn[k], v);
            mx[k] = std::max(mx[k], v);
        }
    int ax = 0;
    for (int k = 1; k < m.dim; ++k)
        if (mx[k] - mn[k] > mx[ax] - mn[ax]) ax = k;
    const size_t parts = (n + T - 1) / T;
    const size_t left = n * (parts / 2) / parts;
    auto key = [&](int c) { return m.cell_pos[3 * (size_t)c + ax]; };
    std::nth_element(ids.begin() + lo, ids.begin() + lo + left, ids.begin() + hi, [&](int a, int b) {
        double ka = key(a), kb = key(b);
        return ka < kb || (ka == kb && a < b);
    });
    rcb(m, ids, lo, lo + left, T, out);
    rcb(m, ids, lo + left, hi, T, out);
}

// RCM order of the cells of one tile (neighbours restricted to the tile).
void rcm_local(const meso_mesh_desc &m, std::vector<int> &cells) {
    const size_t n = cells.size();
    std::vector<int> sorted(cells);
    std::sort(sorted.begin(), sorted.end());
    auto local = [&](int c) -> int {
        auto it = std::lower_bound(sorted.begin(), sorted.end(), c);
        return (it != sorted.end() && *it == c) ? int(it - sorted.begin()) : -1;
    };
    std::vector<int> deg(n, 0);
    for (size_t i = 0; i < n; ++i) {
        int c = sorted[i];
        for (int j = m.cell_nbr_ptr[c]; j < m.cell_nbr_ptr[c + 1]; ++j)
            if (local(m.cell_nbr[j]) >= 0) deg[i]++;
    }
    std::vector<int> by(n);
    std::iota(by.begin(), by.end(), 0);
    std::stable_sort(by.begin(), by.end(), [&](int a, int b) { return deg[a] < deg[b]; });
    std::vector<char> seen(n, 0);
    std::vector<int> order;
    std::vector<int> nb;
    for (int s : by) {
        if (seen[s]) continue;
        size_t head = order.size();
        order.push_back(s);
        seen[s] = 1;
        while (head < order.size()) {
            int i = order[head++];
            int c = sorted[i];
            nb.clear();
            for (int j = m.cell_nbr_ptr[c]; j < m.cell_nbr_ptr[c + 1]; ++j) {
                int l = local(m.cell_nbr[j]);
                if (l >= 0 && !seen[l]) {
                    seen[l] = 1;
                    nb.push_back(l);
                }
            }
            std::stable_sort(nb.begin(), nb.end(), [&](int a, int b) { return deg[a] < deg[b]; });
            order.insert(order.end(), nb.begin(), nb.end());
        }
    }
    std::reverse(order.begin(), order.end());
    for (size_t i = 0; i < n; ++i) cells[i] = sorted[order[i]];
}

}  // namespace

Renumbering renumber_tiled(const meso_mesh_desc &m, int tile_cells, std::vector<int> &tile_sizes) {
    Renumbering r;
    const int C = m.ncell, F = m.nface;
    std::vector<int> ids(C);
    std::iota(ids.begin(), ids.end(), 0);
    std::vector<std::pair<size_t, size_t>> parts;
    rcb(m, ids, 0, (size_t)C, std::max(tile_cells, 1), parts);
    tile_sizes.clear();
    r.cell_new2old.reserve(C);
    for (auto &pr : parts) {
        std::vector<int> cells(ids.begin() + pr.first, ids.begin() + pr.second);
        rcm_local(m, cells);
        r.cell_new2old.insert(r.cell_new2old.end(), cells.begin(), cells.end());
        tile_sizes.push_back((int)cells.size());
    }
    r.cell_old2new.assign(C, 0);
    for (int i = 0; i < C; ++i) r.cell_old2new[r.cell_new2old[i]] = i;
    r.face_new2old.resize(F);
    std::iota(r.face_new2old.begin(), r.face_new2old.end(), 0);
    auto key = [&](int f) {
        return std::make_pair(r.cell_old2new[m.face_cell[2 * f]], r.cell_old2new[m.face_cell[2 * f + 1]]);
    };
    std::stable_sort(r.face_new2old.begin(), r.face_new2old.end(), [&](int a, int b) { return key(a) < key(b); });
    r.face_old2new.assign(F, 0);
    for (int i = 0; i < F; ++i) r.face_old2new[r.face_new2old[i]] = i;
    return r;
}

bool build_tile_plan(const meso_mesh_desc &m, const Renumbering &rn, const std::vector<int> &tile_sizes,
                     int max_slots, int max_gslots, int max_owned, int max_cells, TilePlan &P) {
    const int C = m.ncell, F = m.nface;
    P = TilePlan();
    P.ntile = (int)tile_sizes.size();
    // renumbered adjacency and faces
    auto nbrs = [&](int cn, std::vector<int> &out) {
        out.clear();
        int o = rn.cell_new2old[cn];
        for (int j = m.cell_nbr_ptr[o]; j < m.cell_nbr_ptr[o + 1]; ++j) out.push_back(rn.cell_old2new[m.cell_nbr[j]]);
    };
    std::vector<int> fown(F), fnei(F);
    for (int f = 0; f < F; ++f) {
        int o = rn.face_new2old[f];
        fown[f] = rn.cell_old2new[m.face_cell[2 * o]];
        fnei[f] = rn.cell_old2new[m.face_cell[2 * o + 1]];
    }
    P.face_own_slot.assign(F, 0);
    P.face_nei_slot.assign(F, 0);
    P.tile_fstart.assign(P.ntile + 1, 0);
    std::vector<int> stamp(C, -1), slot_of(C, -1), fstamp(F, -1), flocal(F, 0);
    std::vector<int> nb;
    int cs = 0, fcur = 0;
    for (int t = 0; t < P.ntile; ++t) {
        const int n = tile_sizes[t];
        P.tile_cstart.push_back(cs);
        P.tile_ncell.push_back(n);
        P.tile_slot_ptr.push_back((int)P.slot_cell.size());
        std::vector<int> slots;  // tile cells, then the 1-ring, then the 2-ring
        for (int c = cs; c < cs + n; ++c) {
            stamp[c] = t;
            slot_of[c] = (int)slots.size();
            slots.push_back(c);
        }
        std::vector<int> l1, l2;
        for (int c = cs; c < cs + n; ++c) {
            nbrs(c, nb);
            for (int x : nb)
                if (stamp[x] != t) {
                    stamp[x] = t;
                    l1.push_back(x);
                }
        }
        std::sort(l1.begin(), l1.end());
        // 1-ring cells that are the neighbour of a face the tile owns are reconstructed from, so they
        // need a gradient (and their own neighbours); the rest are only neighbours of tile cells
        std::vector<int> l1a, l1b;
        {
            std::vector<char> up(l1.size(), 0);
            for (int f = fcur; f < F && fown[f] < cs + n; ++f) {
                auto it = std::lower_bound(l1.begin(), l1.end(), fnei[f]);
                if (it != l1.end() && *it == fnei[f]) up[it - l1.begin()] = 1;
            }
            for (size_t k = 0; k < l1.size(); ++k) (up[k] ? l1a : l1b).push_back(l1[k]);
        }
        for (int x : l1a) {
            slot_of[x] = (int)slots.size();
            slots.push_back(x);
        }
        for (int x : l1b) {
            slot_of[x] = (int)slots.size();
            slots.push_back(x);
        }
        for (int c : l1a) {
            nbrs(c, nb);
            for (int x : nb)
                if (stamp[x] != t) {
                    stamp[x] = t;
                    l2.push_back(x);
                }
        }
        std::sort(l2.begin(), l2.end());
        for (int x : l2) {
            slot_of[x] = (int)slots.size();
            slots.push_back(x);
        }
        const int ng = n + (int)l1a.size();
        P.tile_gslots.push_back(ng);
        P.slot_cell.insert(P.slot_cell.end(), slots.begin(), slots.end());
        // gradient stencils of tile + 1-ring slots
        P.tile_gsp_off.push_back((int)P.gs_ptr.size());
        for (int s = 0; s < ng; ++s) {
            P.gs_ptr.push_back((int)P.gs_nbr.size());
            int c = slots[s], o = rn.cell_new2old[c];
            const double *Cx = m.lsq_c + 9 * (size_t)o, *Cy = Cx + 3;
            for (int j = m.cell_nbr_ptr[o]; j < m.cell_nbr_ptr[o + 1]; ++j) {
                int x = rn.cell_old2new[m.cell_nbr[j]];
                const double *dr = m.lsq_dr + 3 * (size_t)j;
                double w = m.lsq_w[j];
                double cx = Cx[0] * dr[0] + Cx[1] * dr[1] + Cx[2] * dr[2];
                double cy = Cy[0] * dr[0] + Cy[1] * dr[1] + Cy[2] * dr[2];
                P.gs_nbr.push_back((uint16_t)slot_of[x]);
                P.gs_ax.push_back((float)(w * cx));
                P.gs_ay.push_back((float)(w * cy));
            }
        }
        P.gs_ptr.push_back((int)P.gs_nbr.size());
        P.max_gentries = std::max(P.max_gentries, P.gs_ptr.back() - P.gs_ptr[P.tile_gsp_off.back()]);
        // owned faces
        P.tile_fstart[t] = fcur;
        while (fcur < F && fown[fcur] < cs + n) {
            P.face_own_slot[fcur] = (uint16_t)slot_of[fown[fcur]];
            P.face_nei_slot[fcur] = (uint16_t)slot_of[fnei[fcur]];
            ++fcur;
        }
        // per cell-face entry: its face in the tile-face list
        const size_t cf0 = P.cf_tf.size();
        const int tf0 = (int)P.tf_face.size();
        P.tile_tf_ptr.push_back(tf0);
        bool tf_ok = true;
        for (int c = cs; c < cs + n; ++c) {
            int o = rn.cell_new2old[c];
            for (int j = m.cell_face_ptr[o]; j < m.cell_face_ptr[o + 1]; ++j) {
                int f = rn.face_old2new[m.cell_face[j]];
                if (fstamp[f] != t) {
                    fstamp[f] = t;
                    flocal[f] = (int)P.tf_face.size() - tf0;
                    P.tf_face.push_back(f);
                }
                tf_ok = tf_ok && flocal[f] < 0x80;
                P.cf_tf.push_back((uint8_t)((flocal[f] & 0x7f) | (fown[f] == c ? 0 : 0x80)));
            }
        }
        P.max_cf = std::max(P.max_cf, (int)(P.cf_tf.size() - cf0));
        P.max_tf = std::max(P.max_tf, tf_ok ? (int)P.tf_face.size() - tf0 : 1 << 20);
        P.max_cells = std::max(P.max_cells, n);
        P.max_slots = std::max(P.max_slots, (int)slots.size());
        P.max_gslots = std::max(P.max_gslots, ng);
        P.max_owned = std::max(P.max_owned, fcur - P.tile_fstart[t]);
        cs += n;
    }
    P.tile_fstart[P.ntile] = fcur;
    P.tile_slot_ptr.push_back((int)P.slot_cell.size());
    P.tile_tf_ptr.push_back((int)P.tf_face.size());
    return fcur == F && P.max_slots <= max_slots && P.max_gslots <= max_gslots && P.max_owned <= max_owned &&
           P.max_cells <= max_cells;
}

}  // namespace meso_host
