// Host-side mesh topology for the sweep: faces, per-cell face slots, the
// neighbour DOF maps used to read upwind traces, and corner coordinates.
//
// This replaces what allium gets from MFEM and igraph at construction time
// (src/sweep.cpp:123-208: face-to-element table, element-to-face table, face
// information).  Faces are matched by sorting their sorted vertex tuples;
// the element with the lower index is the face's element 1, which is the
// element MFEM's face table lists first for a face generated in element order.
#include <algorithm>
#include <array>
#include <climits>
#include <cstring>

#include "internal.h"

namespace allium {
namespace {

const int kQuadCorner[4] = {0, 1, 3, 2};            // corner c0 + 2 c1 -> MFEM local vertex
const int kHexCorner[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // corner c0 + 2 c1 + 4 c2 -> MFEM local vertex

int mfem_vertex(int dim, int c) {
    return dim == 1 ? c : (dim == 2 ? kQuadCorner[c] : kHexCorner[c]);
}

// element corner of face-frame corner m on local face k = 2 axis + side
int face_corner(int dim, int k, int m) {
    const int a = k / 2, s = k % 2;
    int c = 0, j = 0;
    for (int d = 0; d < dim; ++d) {
        const int bit = (d == a) ? s : ((m >> j++) & 1);
        c |= bit << d;
    }
    return c;
}

struct Entry {
    std::array<int, 4> key;
    int e, k;
};

}  // namespace

int build_topology(const allium_mesh_desc& m, int p, Topology& out, std::string& err) {
    const int dim = m.dim, ne = m.num_elements, nc = 1 << dim, nfc = 1 << (dim - 1);
    const int nface = 2 * dim, n1 = p + 1;
    int nf = 1;
    for (int d = 0; d < dim - 1; ++d) nf *= n1;
    auto ev = [&](int e, int c) { return m.element_vertices[(size_t)e * nc + mfem_vertex(dim, c)]; };

    for (long long i = 0; i < (long long)ne * nc; ++i) {
        const int v = m.element_vertices[i];
        if (v < 0 || v >= m.num_vertices) { err = "element vertex index out of range"; return ALLIUM_ERR_MESH; }
    }
    out.corners.resize((size_t)ne * nc * dim);
    for (int e = 0; e < ne; ++e)
        for (int c = 0; c < nc; ++c)
            for (int d = 0; d < dim; ++d)
                out.corners[((size_t)e * nc + c) * dim + d] = m.vertices[(size_t)ev(e, c) * dim + d];

    std::vector<Entry> ent((size_t)ne * nface);
    for (int e = 0; e < ne; ++e)
        for (int k = 0; k < nface; ++k) {
            Entry& x = ent[(size_t)e * nface + k];
            x.key = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
            for (int q = 0; q < nfc; ++q) x.key[q] = ev(e, face_corner(dim, k, q));
            std::sort(x.key.begin(), x.key.begin() + nfc);
            x.e = e; x.k = k;
        }
    std::vector<Entry> sorted = ent;
    std::sort(sorted.begin(), sorted.end(), [](const Entry& a, const Entry& b) {
        if (a.key != b.key) return a.key < b.key;
        if (a.e != b.e) return a.e < b.e;
        return a.k < b.k;
    });

    out.slots.assign((size_t)ne * nface, Slot{-1, -1, 0, 0});
    out.face_e1k1.clear();
    out.nbrmap.assign((size_t)ne * nface * nf, 0);
    out.orient.assign((size_t)ne * nface, FaceOrient{0, 0, 0, 0, 0, 0, 0, 0});
    int nfaces = 0;
    for (size_t i = 0; i < sorted.size();) {
        size_t j = i + 1;
        while (j < sorted.size() && sorted[j].key == sorted[i].key) ++j;
        if (j - i > 2) { err = "a face is shared by more than two elements"; return ALLIUM_ERR_MESH; }
        const Entry& a = sorted[i];
        const int f = nfaces++;
        out.face_e1k1.push_back(a.e);
        out.face_e1k1.push_back(a.k);
        if (j - i == 1) {
            out.slots[(size_t)a.e * nface + a.k] = Slot{f, -1, 0, 0};
        } else {
            const Entry& b = sorted[i + 1];
            if (a.e == b.e) { err = "an element touches itself across a face"; return ALLIUM_ERR_MESH; }
            out.slots[(size_t)a.e * nface + a.k] = Slot{f, b.e, 0, -1};
            out.slots[(size_t)b.e * nface + b.k] = Slot{f, a.e, 1, -1};
            // neighbour DOF maps in both directions
            for (int dir = 0; dir < 2; ++dir) {
                const Entry& s = dir ? b : a;   // self
                const Entry& o = dir ? a : b;   // neighbour
                const int td = dim - 1;
                auto nbr_corner = [&](int ms) {
                    const int v = ev(s.e, face_corner(dim, s.k, ms));
                    for (int mo = 0; mo < nfc; ++mo)
                        if (ev(o.e, face_corner(dim, o.k, mo)) == v) return mo;
                    return -1;
                };
                int bvec[2] = {0, 0}, C[2][2] = {{0, 0}, {0, 0}};
                const int m0 = nbr_corner(0);
                if (m0 < 0) { err = "face vertices do not match"; return ALLIUM_ERR_MESH; }
                for (int jj = 0; jj < td; ++jj) bvec[jj] = (m0 >> jj) & 1;
                for (int c = 0; c < td; ++c) {
                    const int mc = nbr_corner(1 << c);
                    if (mc < 0) { err = "face vertices do not match"; return ALLIUM_ERR_MESH; }
                    for (int jj = 0; jj < td; ++jj) C[jj][c] = ((mc >> jj) & 1) - bvec[jj];
                }
                FaceOrient& fo = out.orient[(size_t)s.e * nface + s.k];
                fo.k2 = (int8_t)o.k;
                fo.b0 = (int8_t)bvec[0]; fo.b1 = (int8_t)bvec[1];
                fo.c00 = (int8_t)C[0][0]; fo.c01 = (int8_t)C[0][1];
                fo.c10 = (int8_t)C[1][0]; fo.c11 = (int8_t)C[1][1];
                const int oa = o.k / 2, os = o.k % 2;
                uint8_t* map = &out.nbrmap[((size_t)s.e * nface + s.k) * nf];
                for (int q = 0; q < nf; ++q) {
                    int t[2] = {0, 0}, r = q;
                    for (int c = 0; c < td; ++c) { t[c] = r % n1; r /= n1; }
                    int sidx[2] = {0, 0};
                    for (int jj = 0; jj < td; ++jj) {
                        int v = bvec[jj] * p;
                        for (int c = 0; c < td; ++c) v += C[jj][c] * t[c];
                        sidx[jj] = v;
                    }
                    int idx = 0, stride = 1, tj = 0;
                    for (int d = 0; d < dim; ++d) {
                        const int id = (d == oa) ? os * p : sidx[tj++];
                        idx += id * stride;
                        stride *= n1;
                    }
                    map[q] = (uint8_t)idx;
                }
            }
        }
        i = j;
    }
    out.nfaces = nfaces;

    // boundary attributes
    for (int bfi = 0; bfi < m.num_boundary_faces; ++bfi) {
        Entry x;
        x.key = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};
        for (int q = 0; q < nfc; ++q) x.key[q] = m.boundary_face_vertices[(size_t)bfi * nfc + q];
        std::sort(x.key.begin(), x.key.begin() + nfc);
        auto it = std::lower_bound(sorted.begin(), sorted.end(), x, [](const Entry& a, const Entry& b) {
            return a.key < b.key;
        });
        if (it == sorted.end() || it->key != x.key) { err = "boundary face is not a face of the mesh"; return ALLIUM_ERR_MESH; }
        Slot& sl = out.slots[(size_t)it->e * nface + it->k];
        if (sl.nbr >= 0) { err = "boundary face is an interior face"; return ALLIUM_ERR_MESH; }
        sl.attr = m.boundary_attributes[bfi];
    }
    return ALLIUM_OK;
}

void mark_reflective(Topology& t, int nface, const std::vector<int>& refl_attrs) {
    t.refl_faces.clear();
    if (refl_attrs.empty()) return;
    for (size_t i = 0; i < t.slots.size(); ++i) {
        Slot& sl = t.slots[i];
        if (sl.nbr != -1) continue;
        if (std::find(refl_attrs.begin(), refl_attrs.end(), sl.attr) == refl_attrs.end()) continue;
        sl.nbr = -2 - (int)t.refl_faces.size();
        t.refl_faces.push_back(sl.face);
    }
    (void)nface;
}

}  // namespace allium
