// ffgpu_numbering.cu -- FreeFEM's node numbering of the scalar P2 space on triangles (host code).
//
// FreeFEM numbers 2D P2 nodes in two steps, and a DOF table handed to the device assembly must
// be that numbering for the matrix pattern to be FreeFEM's:
//  1. ConstructDataFElement::Make (src/femlib/FESpace.cpp:623-877): the node of vertex v is v;
//     edge nodes follow, nv, nv+1, ..., in order of first encounter over (triangle k, local edge
//     j), local edge j being the edge opposite vertex j; a new edge node is given at once to the
//     other triangle holding the edge (Mesh::ElementAdj, fem.cpp:100-260).  Local node order in
//     a triangle: its 3 vertices, then its 3 edges.
//  2. FESpace::renum (src/femlib/gibbs.cpp:1094-1166): the Gibbs-Poole-Stockmeyer profile
//     reduction gibbsa_ (gibbs.cpp:209-433, with gibbsb_, gibbsc_, gibbsd_, gibbst_ and the two
//     heap sorts gibbs1_/gibbs2_) on the node graph of FESpace::gibbsv (gibbs.cpp:1167-1253:
//     two nodes adjacent when a triangle holds both, a node adjacent to itself), applied only
//     when the new profile is not larger than the old one.
// All of it is integer work whose visiting orders decide the result, so the restatement keeps
// the reference's orders, heap-sort comparisons and tie rules; the arrays are 1-based as in the
// reference (slot 0 unused) so that the index arithmetic can be read against it.
#include "ffgpu_internal.cuh"

#include <algorithm>
#include <cstdint>
#include <new>
#include <vector>

namespace ffgpu {
namespace {

typedef int64_t I;

// Heap sort of rec[1..k] by increasing key (gibbs1_/gibbs2_, gibbs.cpp:68-206): the larger child
// is taken on a strict '<' and the sift stops on crit >= child, which fixes the order of equal
// keys.  rec points one slot before the first element.
template <class Key>
void heap_sort(I *rec, I k, const Key &key) {
    if (k <= 1) return;
    I l = k / 2 + 1, r = k;
    for (;;) {
        I v;
        if (l > 1) {
            v = rec[--l];
        } else {
            v = rec[r];
            rec[r] = rec[1];
            if (--r == 1) { rec[1] = v; return; }
        }
        const I crit = key(v);
        I i = l, j = 2 * l;
        while (j <= r) {
            if (j < r && key(rec[j]) < key(rec[j + 1])) ++j;
            if (crit >= key(rec[j])) break;
            rec[i] = rec[j];
            i = j;
            j *= 2;
        }
        rec[i] = v;
    }
}

constexpr I kFree = -1073741824;        // gibbsb_: vertex still to be placed in a level
constexpr I kSeen = -1073741823;        // gibbsb_: placed in a connected piece
constexpr I kOther = -1073741822;       // gibbsb_: vertex of another, unnumbered component

struct Gibbs {
    I n;
    const I *ptv;   // [1..n+1]
    I *adj;         // [1..], neighbour lists sorted in place by degree
    std::vector<I> r, m, lv, nx, ny, nn, wh, wl;

    Gibbs(I n_, const I *ptv_, I *adj_)
        : n(n_), ptv(ptv_), adj(adj_), r(n_ + 1), m(n_ + 1), lv(2 * n_ + 2), nx(n_ + 1), ny(n_ + 1),
          nn(n_ + 1), wh(n_ + 1), wl(n_ + 1) {}

    I deg(I v) const { return ptv[v + 1] - ptv[v]; }

    // Level structure rooted at root (gibbsd_): breadth first, neighbours in list order, over
    // the vertices with r <= 0; level L is lv[lv[L]+1 .. lv[L+1]].  Returns the last level.
    I levels(I root) {
        for (I i = 1; i <= n; ++i)
            if (r[i] < 0) r[i] = 0;
        I top = n, done = n, depth = 0;
        lv[0] = n;
        lv[++top] = root;
        r[root] = -1;
        while (done < top) {
            const I first = done + 1;
            lv[++depth] = top;
            done = top;
            for (I k = first; k <= done; ++k) {
                const I s = lv[k];
                for (I q = ptv[s]; q < ptv[s + 1]; ++q) {
                    const I t = adj[q];
                    if (r[t] == 0) { lv[++top] = t; r[t] = -1; }
                }
            }
        }
        return depth - 1;
    }

    // Level of every vertex in the current structure, -1 outside it (gibbsc_); returns the
    // widest level's size.
    I level_of(std::vector<I> &z, I depth) {
        for (I i = 1; i <= n; ++i) z[i] = -1;
        I widest = 0;
        for (I L = 0; L <= depth; ++L) {
            widest = std::max(widest, lv[L + 1] - lv[L]);
            for (I j = lv[L] + 1; j <= lv[L + 1]; ++j)
                if (lv[j] <= n) z[lv[j]] = L;
        }
        return widest;
    }

    // Width minimisation between the ends x, y of the pseudo-diameter (gibbsb_): vertices on a
    // level consistent from both ends keep it; the other connected pieces, largest first, take
    // the levels from x or from y, whichever keeps the widest level narrower.  Leaves in nn[i]
    // the level of every vertex of the component, -1 for numbered vertices, -2 for vertices of
    // other components.
    void assign_levels(I x, I y) {
        const I cy = level_of(ny, levels(y));
        const I p = levels(x);
        const I cx = level_of(nx, p);
        bool pieces = false;
        for (I i = 1; i <= n; ++i) {
            if (nx[i] + ny[i] == p) r[i] = -nx[i];
            else if (nx[i] >= 0) { pieces = true; r[i] = kFree; }
            else if (r[i] <= 0) r[i] = kOther;
        }
        if (pieces) {
            // connected pieces of the vertices left free, depth first in neighbour order;
            // piece c is lv[lv[c-1]+1 .. lv[c]]
            I top = n, npieces = 0;
            lv[0] = top;
            for (I k = 1; k <= n; ++k) {
                if (r[k] != kFree) continue;
                ++npieces;
                I d = -1, s = k;
                for (;;) {
                    // enter s
                    ++d;
                    wl[d] = ptv[s];
                    wh[d] = ptv[s + 1];
                    lv[++top] = s;
                    r[s] = kSeen;
                    // advance to the next free neighbour, climbing back when a list is spent
                    bool entered = false;
                    while (d >= 0) {
                        if (wl[d] < wh[d]) {
                            const I t = adj[wl[d]++];
                            if (r[t] == kFree) { s = t; entered = true; break; }
                        } else {
                            --d;
                        }
                    }
                    if (!entered) break;
                }
                lv[npieces] = top;
                m[npieces] = npieces;
            }
            heap_sort(m.data(), npieces, [&](I c) { return lv[c] - lv[c - 1]; });
            for (I L = 0; L <= p; ++L) nn[L] = 0;
            for (I i = 1; i <= n; ++i) {
                const I L = -r[i];
                if (L >= 0 && L <= p) ++nn[L];
            }
            for (I k = npieces; k >= 1; --k) {
                const I c = m[k];
                const I i1 = lv[c - 1] + 1, i2 = lv[c];
                for (I L = 0; L <= p; ++L) wh[L] = wl[L] = nn[L];
                for (I i = i1; i <= i2; ++i) {
                    const I s = lv[i];
                    ++wh[nx[s]];
                    ++wl[p - ny[s]];
                }
                I h0 = 0, l0 = 0;
                for (I L = 0; L <= p; ++L) {
                    if (wh[L] != nn[L]) h0 = std::max(wh[L], h0);
                    if (wl[L] != nn[L]) l0 = std::max(wl[L], l0);
                }
                const bool from_x = h0 < l0 || (h0 == l0 && cx <= cy);
                for (I i = i1; i <= i2; ++i) {
                    const I s = lv[i];
                    r[s] = from_x ? -nx[s] : -p + ny[s];
                    ++nn[-r[s]];
                }
            }
        }
        for (I i = 1; i <= n; ++i) {
            if (r[i] > 0) nn[i] = -1;
            else if (r[i] == kOther) nn[i] = -2;
            else nn[i] = -r[i];
        }
    }

    // Cuthill-McKee numbering of the component level by level (gibbst_): option +-1 walks the
    // levels from 0, +-2 from p; inside a level, vertices by the smallest position of an already
    // listed neighbour (3n + degree when none); positive options count up from `next`, negative
    // ones down from next + size.  Advances `next` and returns the profile of the vertices
    // numbered so far.
    I number(I p, I &next, int option) {
        for (I L = 1; L <= p + 1; ++L) lv[L] = 0;
        lv[0] = n;
        for (I i = 1; i <= n; ++i)
            if (nn[i] >= 0) ++lv[nn[i] + 1];
        for (I L = 0; L <= p; ++L) lv[L + 1] += lv[L];
        for (I i = 1; i <= n; ++i)
            if (nn[i] >= 0) {
                const I L = nn[i];
                lv[++lv[L]] = i;
            }
        for (I L = p; L >= 0; --L) lv[L + 1] = lv[L];
        lv[0] = n;
        const I size = lv[p + 1] - lv[0];
        for (I i = 1; i <= n; ++i) m[i] = 3 * n + deg(i);
        const bool up = option == 1 || option == -1;
        for (I s = 0; s <= p; ++s) {
            const I L = up ? s : p - s;
            const I i1 = lv[L] + 1, i2 = lv[L + 1];
            heap_sort(lv.data() + i1 - 1, i2 - i1 + 1, [&](I v) { return m[v]; });
            for (I j = i1; j <= i2; ++j) {
                const I v = lv[j];
                for (I q = ptv[v]; q < ptv[v + 1]; ++q) m[adj[q]] = std::min(m[adj[q]], j);
            }
        }
        I knew = option > 0 ? next : next + size + 1;
        const I step = option > 0 ? 1 : -1;
        next += size;
        for (I s = 0; s <= p; ++s) {
            const I L = up ? s : p - s;
            for (I j = lv[L] + 1; j <= lv[L + 1]; ++j) {
                knew += step;
                r[lv[j]] = knew;
            }
        }
        I pf = 0;
        for (I i = 1; i <= n; ++i) {
            I k = r[i];
            if (k <= 0) continue;
            for (I q = ptv[i]; q < ptv[i + 1]; ++q)
                if (r[adj[q]] > 0) k = std::min(k, r[adj[q]]);
            pf += r[i] - k + 1;
        }
        return pf;
    }

    // gibbsa_: per connected component, root of smallest degree, pseudo-peripheral pair by
    // repeated level structures, level assignment, best of the four numberings.  r[i] = new
    // 1-based number of vertex i; pfold / pfnew the profiles before and after.
    int run(I &pfold, I &pfnew) {
        for (I i = 1; i <= n; ++i)
            heap_sort(adj + ptv[i] - 1, ptv[i + 1] - ptv[i], [&](I v) { return deg(v); });
        for (I i = 1; i <= n; ++i) r[i] = 0;
        I next = 0;
        while (next < n) {
            I y = 0, best = n + 1;
            for (I i = 1; i <= n; ++i)
                if (r[i] <= 0 && deg(i) < best) { best = deg(i); y = i; }
            if (y == 0) return -3;
            I depth = levels(y), x, p;
            for (;;) {
                x = y;
                p = depth;
                I k = 0;
                for (I i = lv[p] + 1; i <= lv[p + 1]; ++i) m[++k] = lv[i];
                heap_sort(m.data(), k, [&](I v) { return deg(v); });
                bool deeper = false;
                for (I i = 1; i <= k; ++i) {
                    y = m[i];
                    depth = levels(y);
                    if (depth > p) { deeper = true; break; }
                }
                if (!deeper) break;
            }
            y = m[1];
            assign_levels(x, y);
            I pf = 1073741824;
            int option = -2;
            const I start = next;
            for (int opt = -2; opt <= 2; ++opt) {
                if (opt == 0) continue;
                next = start;
                const I pf1 = number(p, next, opt);
                if (pf1 < pf) { pf = pf1; option = opt; }
            }
            next = start;
            number(p, next, option);
        }
        // profiles before and after, kept in units of 1e9 past 1e9 as the reference does
        const I big = 1000000000;
        I po = 0, pn = 0, po1 = 0, pn1 = 0;
        for (I i = 1; i <= n; ++i) {
            I lo_old = i, lo_new = r[i];
            for (I q = ptv[i]; q < ptv[i + 1]; ++q) {
                lo_old = std::min(lo_old, adj[q]);
                lo_new = std::min(lo_new, r[adj[q]]);
            }
            po += i - lo_old + 1;
            pn += r[i] - lo_new + 1;
            if (po > big) { po1 += po / big; po %= big; }
            if (pn > big) { pn1 += pn / big; pn %= big; }
        }
        if (po1 || pn1) {
            if (po1 == pn1) {
                pn = pn1 * 10 + (pn >= po);
                po = po1 * 10 + (pn <= po);
            } else {
                pn = pn1;
                po = po1;
            }
        }
        pfold = po;
        pfnew = pn;
        return 0;
    }
};

}  // namespace
}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

int ffgpu_gibbs_renumber(int64_t n, const int64_t *ptvois, int64_t *vois, int64_t *r, int64_t *pfold,
                         int64_t *pfnew) {
    FFGPU_CHECK(n >= 1 && ptvois && vois && r && pfold && pfnew, FFGPU_EINVAL,
                "ffgpu_gibbs_renumber: bad argument");
    FFGPU_CHECK(ptvois[0] == 1, FFGPU_EINVAL, "ffgpu_gibbs_renumber: ptvois must start at 1");
    for (int64_t i = 0; i < n; ++i)
        FFGPU_CHECK(ptvois[i + 1] >= ptvois[i], FFGPU_EINVAL, "ffgpu_gibbs_renumber: ptvois not ascending");
    for (int64_t q = 0; q < ptvois[n] - 1; ++q)
        FFGPU_CHECK(vois[q] >= 1 && vois[q] <= n, FFGPU_EINVAL, "ffgpu_gibbs_renumber: neighbour %lld out of range",
                    (long long)vois[q]);
    try {
        // 1-based views: ptv[i] = ptvois[i-1], adj[q] = vois[q-1]
        Gibbs g(n, ptvois - 1, vois - 1);
        I po = 0, pn = 0;
        const int rc = g.run(po, pn);
        FFGPU_CHECK(rc == 0, FFGPU_EINVAL, "ffgpu_gibbs_renumber: no root found");
        for (int64_t i = 0; i < n; ++i) r[i] = g.r[i + 1];
        *pfold = po;
        *pfnew = pn;
    } catch (const std::bad_alloc &) {
        set_error("ffgpu_gibbs_renumber: out of host memory");
        return FFGPU_ENOMEM;
    }
    return FFGPU_OK;
}

int ffgpu_number_p2_2d(int nv, int nt, const int32_t *elems, int32_t *nodes, int *nnodes) {
    FFGPU_CHECK(nv > 0 && nt > 0 && elems && nodes && nnodes, FFGPU_EINVAL, "ffgpu_number_p2_2d: bad argument");
    try {
        for (int64_t k = 0; k < 3 * (int64_t)nt; ++k)
            FFGPU_CHECK(elems[k] >= 0 && elems[k] < nv, FFGPU_EINVAL,
                        "ffgpu_number_p2_2d: triangle %lld lists vertex %d outside [0, %d)", (long long)(k / 3),
                        elems[k], nv);
        // edges as (lower vertex, upper vertex, triangle, local edge), sorted: the triangles
        // sharing an edge are neighbours in the list
        struct Slot { int32_t a, b, t, j; };
        std::vector<Slot> e((size_t)nt * 3);
        for (int t = 0; t < nt; ++t)
            for (int j = 0; j < 3; ++j) {
                const int32_t p = elems[3 * (int64_t)t + (j + 1) % 3], q = elems[3 * (int64_t)t + (j + 2) % 3];
                e[3 * (size_t)t + j] = Slot{std::min(p, q), std::max(p, q), t, j};
            }
        std::sort(e.begin(), e.end(), [](const Slot &x, const Slot &y) {
            return x.a != y.a ? x.a < y.a : (x.b != y.b ? x.b < y.b : (x.t != y.t ? x.t < y.t : x.j < y.j));
        });
        std::vector<int64_t> partner((size_t)nt * 3, -1);   // slot 3t+j -> slot of the other triangle
        for (size_t s = 0; s < e.size();) {
            size_t u = s + 1;
            while (u < e.size() && e[u].a == e[s].a && e[u].b == e[s].b) ++u;
            FFGPU_CHECK(u - s <= 2, FFGPU_EMESH, "ffgpu_number_p2_2d: edge (%d, %d) shared by %d triangles", e[s].a,
                        e[s].b, (int)(u - s));
            if (u - s == 2) {
                partner[3 * (size_t)e[s].t + e[s].j] = 3 * (int64_t)e[s + 1].t + e[s + 1].j;
                partner[3 * (size_t)e[s + 1].t + e[s + 1].j] = 3 * (int64_t)e[s].t + e[s].j;
            }
            s = u;
        }
        // step 1: vertex nodes, then edge nodes by first encounter
        std::vector<int32_t> node((size_t)nt * 6, -1);
        int64_t nn = nv;
        for (int t = 0; t < nt; ++t) {
            for (int j = 0; j < 3; ++j) node[6 * (size_t)t + j] = elems[3 * (int64_t)t + j];
            for (int j = 0; j < 3; ++j) {
                int32_t &mine = node[6 * (size_t)t + 3 + j];
                if (mine >= 0) continue;
                const int64_t o = partner[3 * (size_t)t + j];
                if (o >= 0) node[6 * (size_t)(o / 3) + 3 + o % 3] = (int32_t)nn;
                mine = (int32_t)nn++;
            }
        }
        FFGPU_CHECK(nn <= INT32_MAX, FFGPU_EMESH, "ffgpu_number_p2_2d: too many nodes");
        const int64_t n = nn;
        // step 2: the node graph of FESpace::gibbsv -- for each node, the triangles holding it in
        // ascending order, their nodes in local order, first occurrence kept (the node itself
        // included); at most 20 neighbours per node on average, else no renumbering
        std::vector<int64_t> ptv(n + 2, 0);
        for (size_t k = 0; k < node.size(); ++k) ++ptv[node[k] + 1];
        for (int64_t i = 0; i < n; ++i) ptv[i + 1] += ptv[i];
        std::vector<int32_t> tri(node.size());
        {
            std::vector<int64_t> fill(ptv.begin(), ptv.end() - 1);
            for (int t = 0; t < nt; ++t)
                for (int j = 0; j < 6; ++j) tri[fill[node[6 * (size_t)t + j]]++] = t;
        }
        const int64_t cap = 20 * n;
        std::vector<int64_t> gptr(n + 1), gadj;
        std::vector<int64_t> mark(n, -1);
        bool fits = true;
        gadj.reserve((size_t)std::min<int64_t>(cap, 12 * n));
        for (int64_t i = 0; i < n && fits; ++i) {
            gptr[i] = (int64_t)gadj.size() + 1;
            for (int64_t q = ptv[i]; q < ptv[i + 1] && fits; ++q) {
                const int t = tri[q];
                for (int j = 0; j < 6; ++j) {
                    const int32_t v = node[6 * (size_t)t + j];
                    if (mark[v] == i) continue;
                    mark[v] = i;
                    if ((int64_t)gadj.size() >= cap) { fits = false; break; }
                    gadj.push_back(v + 1);
                }
            }
        }
        gptr[n] = (int64_t)gadj.size() + 1;
        if (fits && (int64_t)gadj.size() > n) {
            std::vector<int64_t> r(n);
            int64_t po = 0, pn = 0;
            FFGPU_TRY(ffgpu_gibbs_renumber(n, gptr.data(), gadj.data(), r.data(), &po, &pn));
            if (pn <= po)
                for (size_t k = 0; k < node.size(); ++k) node[k] = (int32_t)(r[node[k]] - 1);
        }
        std::copy(node.begin(), node.end(), nodes);
        *nnodes = (int)n;
    } catch (const std::bad_alloc &) {
        set_error("ffgpu_number_p2_2d: out of host memory");
        return FFGPU_ENOMEM;
    }
    return FFGPU_OK;
}

}  // extern "C"
