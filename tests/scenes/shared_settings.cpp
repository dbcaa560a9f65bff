// Host-side mirror of SoftBodySharedSettings (see shared_settings.h).
//
// Byte-identical output with the reference requires the same handling of equal keys, so the sort
// and heap routines below implement the same published algorithms the reference uses, with the
// same parameters:
//   * quicksort with a ninther pivot, Hoare partitioning, recursion into the smaller side and an
//     insertion-sort cutoff at 32 elements (Jolt/Core/QuickSort.h, Jolt/Core/InsertionSort.h).
//     It is not stable; the order of equal edges decides which triangle is "first" at a shared edge
//     and therefore the vertex order inside dihedral bend and shear constraints.
//   * a binary max-heap push/pop (Jolt/Core/BinaryHeap.h) driving Dijkstra's search for the closest
//     kinematic vertex; the pop order of equal distances decides which kinematic vertex an LRA
//     tether attaches to.
// Compile with -ffp-contract=off.

#include <stdexcept>
#include "shared_settings.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "fmath.h"

namespace jsb {
namespace host {

namespace {

// ---- insertion sort used below the quicksort cutoff --------------------------------------------
template <class T, class Less>
void insertion_sort(T *first, T *last, Less less) {
    if (first == last) return;
    for (T *i = first + 1; i != last; ++i) {
        T x = *i;
        if (less(x, *first)) {
            for (T *j = i; j != first; --j) *j = *(j - 1);
            *first = x;
        } else {
            T *j = i;
            for (T *prev = j - 1; less(x, *prev); j = prev, --prev) *j = *prev;
            *j = x;
        }
    }
}

// Orders *a, *b, *c so that *b holds the median of the three.
template <class T, class Less>
void median3(T *a, T *b, T *c, Less less) {
    if (less(*b, *a)) std::swap(*a, *b);
    if (less(*c, *a)) std::swap(*a, *c);
    if (less(*c, *b)) std::swap(*b, *c);
}

// Tukey's ninther: medians of three triples spread over [first, last], then their median into mid.
template <class T, class Less>
void ninther(T *first, T *mid, T *last, Less less) {
    ptrdiff_t step = (last - first) >> 3;
    ptrdiff_t step2 = step << 1;
    T *m1 = first + step;
    median3(first, m1, first + step2, less);
    median3(mid - step, mid, mid + step, less);
    T *m3 = last - step;
    median3(last - step2, m3, last, less);
    median3(m1, mid, m3, less);
}

template <class T, class Less>
void quick_sort(T *begin, T *end, Less less) {
    for (;;) {
        ptrdiff_t n = end - begin;
        if (n < 2) return;
        if (n <= 32) {
            insertion_sort(begin, end, less);
            return;
        }
        T *mid = begin + ((n - 1) >> 1);
        ninther(begin, mid, end - 1, less);
        T pivot = *mid;
        T *i = begin;
        T *j = end;
        for (;;) {
            while (less(*i, pivot)) ++i;
            do
                --j;
            while (less(pivot, *j));
            if (i >= j) break;
            std::swap(*i, *j);
            ++i;
        }
        ++j;
        if (j - begin < end - j) {
            quick_sort(begin, j, less);
            begin = j;
        } else {
            quick_sort(j, end, less);
            end = j;
        }
    }
}

template <class T, class Less>
void quick_sort(std::vector<T> &v, Less less) {
    if (!v.empty()) quick_sort(v.data(), v.data() + v.size(), less);
}

// ---- binary max-heap (pred(a, b) == "a ranks below b") ------------------------------------------
template <class T, class Pred>
void heap_push(std::vector<T> &h, Pred pred) {
    ptrdiff_t cur = ptrdiff_t(h.size()) - 1;
    while (cur > 0) {
        ptrdiff_t parent = (cur - 1) >> 1;
        if (pred(h[parent], h[cur])) {
            std::swap(h[parent], h[cur]);
            cur = parent;
        } else
            break;
    }
}

template <class T, class Pred>
void heap_pop(std::vector<T> &h, Pred pred) {  // moves the top to h.back()
    std::swap(h.back(), h.front());
    ptrdiff_t count = ptrdiff_t(h.size()) - 1;
    ptrdiff_t largest = 0;
    for (;;) {
        ptrdiff_t child = (largest << 1) + 1;
        if (child >= count) break;
        ptrdiff_t prev = largest;
        if (pred(h[largest], h[child])) largest = child;
        ++child;
        if (child < count && pred(h[largest], h[child])) largest = child;
        if (prev == largest) break;
        std::swap(h[prev], h[largest]);
    }
}

inline F3 pos_of(const SoftBodySharedSettings::Vertex &v) { return {v.mPosition[0], v.mPosition[1], v.mPosition[2]}; }

template <class T>
void put(std::string &out, const T &v) {
    out.append(reinterpret_cast<const char *>(&v), sizeof(T));
}

template <class T>
void put_array(std::string &out, const std::vector<T> &v) {
    uint32_t n = uint32_t(v.size());
    put(out, n);
    if (n) out.append(reinterpret_cast<const char *>(v.data()), sizeof(T) * v.size());
}

}  // namespace

uint32_t SoftBodySharedSettings::DihedralBend::GetMinVertexIndex() const {
    return std::min(std::min(mVertex[0], mVertex[1]), std::min(mVertex[2], mVertex[3]));
}
uint32_t SoftBodySharedSettings::Volume::GetMinVertexIndex() const {
    return std::min(std::min(mVertex[0], mVertex[1]), std::min(mVertex[2], mVertex[3]));
}

// SoftBodySharedSettings.cpp:110-187
void SoftBodySharedSettings::CalculateClosestKinematic() {
    if (!mClosestKinematic.empty()) return;
    mClosestKinematic.resize(mVertices.size());
    std::vector<std::vector<uint32_t>> adjacency(mVertices.size());
    for (const Edge &e : mEdgeConstraints) {
        adjacency[e.mVertex[0]].push_back(e.mVertex[1]);
        adjacency[e.mVertex[1]].push_back(e.mVertex[0]);
    }
    struct Open {
        uint32_t vertex;
        float distance;
    };
    // "a ranks below b" when a is farther: the heap top is the nearest open vertex
    auto below = [](const Open &a, const Open &b) { return a.distance > b.distance; };
    std::vector<Open> open;
    for (uint32_t v = 0; v < mVertices.size(); ++v)
        if (mVertices[v].mInvMass == 0.0f) {
            mClosestKinematic[v].mVertex = v;
            mClosestKinematic[v].mHops = 0;
            mClosestKinematic[v].mDistance = 0.0f;
            open.push_back({v, 0.0f});
            heap_push(open, below);
        }
    while (!open.empty()) {
        heap_pop(open, below);
        Open cur = open.back();
        open.pop_back();
        for (uint32_t v : adjacency[cur.vertex]) {
            float d = cur.distance + length(pos_of(mVertices[v]) - pos_of(mVertices[cur.vertex]));
            if (d < mClosestKinematic[v].mDistance) {
                mClosestKinematic[v].mVertex = mClosestKinematic[cur.vertex].mVertex;
                mClosestKinematic[v].mHops = mClosestKinematic[cur.vertex].mHops + 1;
                mClosestKinematic[v].mDistance = d;
                open.push_back({v, d});
                heap_push(open, below);
            }
        }
    }
}

// SoftBodySharedSettings.cpp:189-369
void SoftBodySharedSettings::CreateConstraints(const VertexAttributes *attrs, uint32_t n_attrs, EBendType bend_type,
                                               float angle_tolerance) {
    struct EdgeRef {
        uint32_t v[2];
        uint32_t edge_idx;  // face * 3 + corner
    };
    std::vector<EdgeRef> edges;
    edges.reserve(mFaces.size() * 3);
    for (size_t fi = 0; fi < mFaces.size(); ++fi) {
        const Face &f = mFaces[fi];
        for (int i = 0; i < 3; ++i) {
            uint32_t a = f.mVertex[i], b = f.mVertex[(i + 1) % 3];
            edges.push_back({{std::min(a, b), std::max(a, b)}, uint32_t(fi) * 3 + uint32_t(i)});
        }
    }
    quick_sort(edges, [](const EdgeRef &l, const EdgeRef &r) {
        return l.v[0] < r.v[0] || (l.v[0] == r.v[0] && l.v[1] < r.v[1]);
    });

    auto add_edge = [this](uint32_t v1, uint32_t v2, float c1, float c2) {
        if ((mVertices[v1].mInvMass > 0.0f || mVertices[v2].mInvMass > 0.0f) && c1 < FLT_MAX && c2 < FLT_MAX) {
            Edge e;
            e.mVertex[0] = v1;
            e.mVertex[1] = v2;
            e.mCompliance = 0.5f * (c1 + c2);
            e.mRestLength = length(pos_of(mVertices[v2]) - pos_of(mVertices[v1]));
            mEdgeConstraints.push_back(e);
        }
    };
    auto attr = [attrs, n_attrs](uint32_t v) -> const VertexAttributes & { return attrs[std::min(v, n_attrs - 1)]; };

    // Sin/Cos of the tolerance only feed threshold tests on near-planar, near-square quads
    float s = float(std::sin(double(angle_tolerance)));
    float c = float(std::cos(double(angle_tolerance)));
    float sq_sin_tolerance = s * s;
    float sq_cos_tolerance = c * c;

    mEdgeConstraints.clear();
    mEdgeConstraints.reserve(edges.size());
    for (size_t i = 0; i < edges.size(); ++i) {
        const EdgeRef e0 = edges[i];
        const VertexAttributes &a0 = attr(e0.v[0]);
        const VertexAttributes &a1 = attr(e0.v[1]);
        bool is_shear = false;
        for (size_t j = i + 1; j < edges.size(); ++j) {
            const EdgeRef &e1 = edges[j];
            if (e0.v[0] == e1.v[0] && e0.v[1] == e1.v[1]) {
                const Face &f0 = mFaces[e0.edge_idx / 3];
                const Face &f1 = mFaces[e1.edge_idx / 3];
                uint32_t opp0 = f0.mVertex[(e0.edge_idx + 2) % 3];
                uint32_t opp1 = f1.mVertex[(e1.edge_idx + 2) % 3];
                const VertexAttributes &ao0 = attr(opp0);
                const VertexAttributes &ao1 = attr(opp1);
                if (opp0 == opp1) continue;
                F3 p00 = pos_of(mVertices[f0.mVertex[0]]);
                F3 n0 = cross(pos_of(mVertices[f0.mVertex[2]]) - p00, pos_of(mVertices[f0.mVertex[1]]) - p00);
                F3 p10 = pos_of(mVertices[f1.mVertex[0]]);
                F3 n1 = cross(pos_of(mVertices[f1.mVertex[2]]) - p10, pos_of(mVertices[f1.mVertex[1]]) - p10);
                float n0n1 = dot(n0, n1);
                if (n0n1 > 0.0f && n0n1 * n0n1 > sq_cos_tolerance * length_sq(n0) * length_sq(n1)) {
                    F3 base = pos_of(mVertices[e0.v[0]]);
                    F3 d0 = pos_of(mVertices[opp0]) - base;
                    F3 d1 = pos_of(mVertices[opp1]) - base;
                    float dd = dot(d0, d1);
                    if (dd * dd < sq_sin_tolerance * length_sq(d0) * length_sq(d1)) {
                        add_edge(opp0, opp1, ao0.shear_compliance, ao1.shear_compliance);
                        is_shear = true;
                    }
                }
                switch (bend_type) {
                    case EBendType::None:
                        break;
                    case EBendType::Distance:
                        if (!is_shear) add_edge(opp0, opp1, a0.bend_compliance, a1.bend_compliance);
                        break;
                    case EBendType::Dihedral:
                        if ((mVertices[opp0].mInvMass > 0.0f || mVertices[opp1].mInvMass > 0.0f) && a0.bend_compliance < FLT_MAX &&
                            a1.bend_compliance < FLT_MAX) {
                            DihedralBend b;
                            b.mVertex[0] = e0.v[0];
                            b.mVertex[1] = e0.v[1];
                            b.mVertex[2] = opp0;
                            b.mVertex[3] = opp1;
                            b.mCompliance = 0.5f * (a0.bend_compliance + a1.bend_compliance);
                            mDihedralBendConstraints.push_back(b);
                        }
                        break;
                }
            } else {
                i = j - 1;
                break;
            }
        }
        add_edge(e0.v[0], e0.v[1], is_shear ? a0.shear_compliance : a0.compliance, is_shear ? a1.shear_compliance : a1.compliance);
    }
    mEdgeConstraints.shrink_to_fit();

    CalculateBendConstraintConstants();

    bool has_lra = false;
    for (uint32_t k = 0; k < n_attrs; ++k)
        if (attrs[k].lra_type != ELRAType::None) {
            has_lra = true;
            break;
        }
    if (has_lra) {
        CalculateClosestKinematic();
        for (uint32_t v = 0; v < uint32_t(mVertices.size()); ++v)
            if (mVertices[v].mInvMass > 0.0f) {
                uint32_t closest = mClosestKinematic[v].mVertex;
                if (closest == 0xffffffff) continue;
                const VertexAttributes &va = attr(v);
                LRA l;
                l.mVertex[0] = closest;
                l.mVertex[1] = v;
                switch (va.lra_type) {
                    case ELRAType::None:
                        continue;
                    case ELRAType::EuclideanDistance:
                        l.mMaxDistance = va.lra_max_distance_multiplier * length(pos_of(mVertices[closest]) - pos_of(mVertices[v]));
                        break;
                    case ELRAType::GeodesicDistance:
                        l.mMaxDistance = va.lra_max_distance_multiplier * mClosestKinematic[v].mDistance;
                        break;
                }
                mLRAConstraints.push_back(l);
            }
    }
}

void SoftBodySharedSettings::CalculateEdgeLengths() {  // SoftBodySharedSettings.cpp:371-379
    for (Edge &e : mEdgeConstraints) e.mRestLength = length(pos_of(mVertices[e.mVertex[1]]) - pos_of(mVertices[e.mVertex[0]]));
}

void SoftBodySharedSettings::CalculateLRALengths(float mult) {  // :483-491
    for (LRA &l : mLRAConstraints) l.mMaxDistance = mult * length(pos_of(mVertices[l.mVertex[1]]) - pos_of(mVertices[l.mVertex[0]]));
}

void SoftBodySharedSettings::CalculateBendConstraintConstants() {  // :493-532
    for (DihedralBend &b : mDihedralBendConstraints) {
        F3 x0 = pos_of(mVertices[b.mVertex[0]]), x1 = pos_of(mVertices[b.mVertex[1]]);
        F3 x2 = pos_of(mVertices[b.mVertex[2]]), x3 = pos_of(mVertices[b.mVertex[3]]);
        F3 e0 = x1 - x0, e1 = x2 - x0, e2 = x3 - x0;
        F3 n1 = cross(e0, e1);
        F3 n2 = cross(e2, e0);
        float denom = std::sqrt(length_sq(n1) * length_sq(n2));
        if (denom < 1.0e-12f)
            b.mInitialAngle = 0.0f;
        else
            b.mInitialAngle = sign_of(dot(cross(n2, n1), e0)) * acos_approximate(dot(n1, n2) / denom);
    }
}

void SoftBodySharedSettings::CalculateVolumeConstraintVolumes() {  // :534-554
    for (Volume &v : mVolumeConstraints) {
        F3 x1 = pos_of(mVertices[v.mVertex[0]]), x2 = pos_of(mVertices[v.mVertex[1]]);
        F3 x3 = pos_of(mVertices[v.mVertex[2]]), x4 = pos_of(mVertices[v.mVertex[3]]);
        F3 x1x2 = x2 - x1, x1x3 = x3 - x1, x1x4 = x4 - x1;
        v.mSixRestVolume = std::fabs(dot(cross(x1x2, x1x3), x1x4));
    }
}

// SoftBodySharedSettings.cpp:613-1182, restricted to the constraint types the GPU path supports
// (edges, LRA, dihedral bends, volumes; no rods or skinned constraints).
void SoftBodySharedSettings::Optimize() {
    mUpdateGroups.clear();
    const uint32_t nv = uint32_t(mVertices.size());

    struct Link {
        uint32_t vertex;
        uint32_t count;
    };
    std::vector<std::vector<Link>> links(nv);
    auto connect = [&links](uint32_t a, uint32_t b) {
        for (int pass = 0; pass < 2; ++pass) {
            bool found = false;
            for (Link &l : links[a])
                if (l.vertex == b) {
                    l.count++;
                    found = true;
                    break;
                }
            if (!found) links[a].push_back({b, 1});
            std::swap(a, b);
        }
    };
    for (const Edge &c : mEdgeConstraints) connect(c.mVertex[0], c.mVertex[1]);
    for (const LRA &c : mLRAConstraints) connect(c.mVertex[0], c.mVertex[1]);
    auto connect4 = [&connect](const uint32_t *v) {
        connect(v[0], v[1]);
        connect(v[0], v[2]);
        connect(v[0], v[3]);
        connect(v[1], v[2]);
        connect(v[1], v[3]);
        connect(v[2], v[3]);
    };
    for (const DihedralBend &c : mDihedralBendConstraints) connect4(c.mVertex);
    for (const Volume &c : mVolumeConstraints) connect4(c.mVertex);

    const uint32_t kBatch = 256;  // SoftBodyUpdateContext::cVertexConstraintBatch
    std::vector<int> group_of(nv, -1);
    int cur_group = 0;
    std::vector<uint32_t> members;
    for (;;) {
        // bounds of the ungrouped vertices
        F3 bmin = {FLT_MAX, FLT_MAX, FLT_MAX}, bmax = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (uint32_t i = 0; i < nv; ++i)
            if (group_of[i] == -1) {
                F3 p = pos_of(mVertices[i]);
                bmin = {bmin.x < p.x ? bmin.x : p.x, bmin.y < p.y ? bmin.y : p.y, bmin.z < p.z ? bmin.z : p.z};
                bmax = {bmax.x > p.x ? bmax.x : p.x, bmax.y > p.y ? bmax.y : p.y, bmax.z > p.z ? bmax.z : p.z};
            }
        if (!(bmin.x <= bmax.x && bmin.y <= bmax.y && bmin.z <= bmax.z)) break;
        F3 size = bmax - bmin;
        uint32_t max_axis = size.x > size.y ? (size.z > size.x ? 2 : 0) : (size.z > size.y ? 2 : 1);
        uint32_t min_axis = size.x < size.y ? (size.z < size.x ? 2 : 0) : (size.z < size.y ? 2 : 1);
        if (min_axis == max_axis) min_axis = (min_axis + 1) % 3;
        uint32_t mid_axis = 3 - min_axis - max_axis;

        uint32_t seed = UINT32_MAX;
        float best[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
        for (uint32_t i = 0; i < nv; ++i)
            if (group_of[i] == -1) {
                const float *p = mVertices[i].mPosition;
                float a = p[max_axis], m = p[mid_axis], n = p[min_axis];
                if (a < best[max_axis] || (a == best[max_axis] && (m < best[mid_axis] || (m == best[mid_axis] && n < best[min_axis])))) {
                    best[0] = p[0];
                    best[1] = p[1];
                    best[2] = p[2];
                    seed = i;
                }
            }
        if (seed == UINT32_MAX) break;
        members.push_back(seed);
        group_of[seed] = cur_group;

        for (;;) {
            uint32_t best_v = UINT32_MAX, best_links = 0;
            float best_d2 = FLT_MAX;
            F3 first = pos_of(mVertices[members.front()]);
            for (size_t k = 0; k < members.size(); ++k)
                for (const Link &l : links[members[k]]) {
                    uint32_t v = l.vertex;
                    if (group_of[v] != -1) continue;
                    uint32_t n_links = 0;
                    for (const Link &l2 : links[v])
                        if (group_of[l2.vertex] == cur_group) n_links += l2.count;
                    float d2 = length_sq(pos_of(mVertices[v]) - first);
                    if (best_v == UINT32_MAX || n_links > best_links || (n_links == best_links && d2 < best_d2)) {
                        best_v = v;
                        best_links = n_links;
                        best_d2 = d2;
                    }
                }
            if (best_v != UINT32_MAX) {
                members.push_back(best_v);
                group_of[best_v] = cur_group;
            }
            if (members.size() >= kBatch || (members.size() > kBatch / 2 && best_v == UINT32_MAX)) {
                members.clear();
                cur_group++;
                break;
            }
            if (best_v == UINT32_MAX) break;
        }
    }
    if (members.size() > kBatch / 2) ++cur_group;
    members.clear();
    links.clear();

    struct Group {
        std::vector<uint32_t> edges, lras, bends, volumes;
        uint32_t size() const { return uint32_t(edges.size() + lras.size() + bends.size() + volumes.size()); }
    };
    std::vector<Group> groups(size_t(cur_group) + 1);
    Group &np = groups.back();
    for (size_t i = 0; i < mEdgeConstraints.size(); ++i) {
        int g1 = group_of[mEdgeConstraints[i].mVertex[0]], g2 = group_of[mEdgeConstraints[i].mVertex[1]];
        (g1 == g2 ? groups[g1] : groups.back()).edges.push_back(uint32_t(i));
    }
    for (size_t i = 0; i < mLRAConstraints.size(); ++i) {
        int g1 = group_of[mLRAConstraints[i].mVertex[0]], g2 = group_of[mLRAConstraints[i].mVertex[1]];
        (g1 == g2 ? groups[g1] : groups.back()).lras.push_back(uint32_t(i));
    }
    for (size_t i = 0; i < mDihedralBendConstraints.size(); ++i) {
        const uint32_t *v = mDihedralBendConstraints[i].mVertex;
        int g1 = group_of[v[0]], g2 = group_of[v[1]], g3 = group_of[v[2]], g4 = group_of[v[3]];
        (g1 == g2 && g1 == g3 && g1 == g4 ? groups[g1] : groups.back()).bends.push_back(uint32_t(i));
    }
    for (size_t i = 0; i < mVolumeConstraints.size(); ++i) {
        const uint32_t *v = mVolumeConstraints[i].mVertex;
        int g1 = group_of[v[0]], g2 = group_of[v[1]], g3 = group_of[v[2]], g4 = group_of[v[3]];
        (g1 == g2 && g1 == g3 && g1 == g4 ? groups[g1] : groups.back()).volumes.push_back(uint32_t(i));
    }
    (void)np;

    // Parallel groups big to small. The sort is unstable, so sort an index permutation with the
    // same algorithm (the permutation depends only on comparisons and swaps).
    {
        std::vector<uint32_t> order(groups.size() - 1);
        for (size_t i = 0; i < order.size(); ++i) order[i] = uint32_t(i);
        std::vector<uint32_t> sizes(groups.size());
        for (size_t i = 0; i < groups.size(); ++i) sizes[i] = groups[i].size();
        quick_sort(order, [&sizes](uint32_t a, uint32_t b) { return sizes[a] > sizes[b]; });
        std::vector<Group> sorted;
        sorted.reserve(groups.size());
        for (uint32_t g : order) sorted.push_back(std::move(groups[g]));
        sorted.push_back(std::move(groups.back()));
        groups.swap(sorted);
    }

    CalculateClosestKinematic();
    const auto &ck = mClosestKinematic;
    for (Group &g : groups) {
        quick_sort(g.edges, [&](uint32_t l, uint32_t r) {
            const Edge &e1 = mEdgeConstraints[l], &e2 = mEdgeConstraints[r];
            float d1 = std::min(ck[e1.mVertex[0]].mDistance, ck[e1.mVertex[1]].mDistance);
            float d2 = std::min(ck[e2.mVertex[0]].mDistance, ck[e2.mVertex[1]].mDistance);
            if (d1 != d2) return d1 < d2;
            uint32_t m1 = e1.GetMinVertexIndex(), m2 = e2.GetMinVertexIndex();
            if (m1 != m2) return m1 < m2;
            return l < r;
        });
        quick_sort(g.lras, [&](uint32_t l, uint32_t r) {
            const LRA &a = mLRAConstraints[l], &b = mLRAConstraints[r];
            if (a.mMaxDistance != b.mMaxDistance) return a.mMaxDistance > b.mMaxDistance;
            uint32_t m1 = a.GetMinVertexIndex(), m2 = b.GetMinVertexIndex();
            if (m1 != m2) return m1 < m2;
            return l < r;
        });
        auto min4 = [&ck](const uint32_t *v) {
            return std::min(std::min(ck[v[0]].mDistance, ck[v[1]].mDistance), std::min(ck[v[2]].mDistance, ck[v[3]].mDistance));
        };
        quick_sort(g.bends, [&](uint32_t l, uint32_t r) {
            const DihedralBend &b1 = mDihedralBendConstraints[l], &b2 = mDihedralBendConstraints[r];
            float d1 = min4(b1.mVertex), d2 = min4(b2.mVertex);
            if (d1 != d2) return d1 < d2;
            uint32_t m1 = b1.GetMinVertexIndex(), m2 = b2.GetMinVertexIndex();
            if (m1 != m2) return m1 < m2;
            return l < r;
        });
        quick_sort(g.volumes, [&](uint32_t l, uint32_t r) {
            const Volume &v1 = mVolumeConstraints[l], &v2 = mVolumeConstraints[r];
            float d1 = min4(v1.mVertex), d2 = min4(v2.mVertex);
            if (d1 != d2) return d1 < d2;
            uint32_t m1 = v1.GetMinVertexIndex(), m2 = v2.GetMinVertexIndex();
            if (m1 != m2) return m1 < m2;
            return l < r;
        });
    }

    std::vector<Edge> old_edges;
    old_edges.swap(mEdgeConstraints);
    std::vector<LRA> old_lras;
    old_lras.swap(mLRAConstraints);
    std::vector<DihedralBend> old_bends;
    old_bends.swap(mDihedralBendConstraints);
    std::vector<Volume> old_volumes;
    old_volumes.swap(mVolumeConstraints);
    for (const Group &g : groups) {
        for (uint32_t i : g.edges) mEdgeConstraints.push_back(old_edges[i]);
        for (uint32_t i : g.lras) mLRAConstraints.push_back(old_lras[i]);
        for (uint32_t i : g.bends) mDihedralBendConstraints.push_back(old_bends[i]);
        for (uint32_t i : g.volumes) mVolumeConstraints.push_back(old_volumes[i]);
        UpdateGroup ug;
        ug.mEdgeEndIndex = uint32_t(mEdgeConstraints.size());
        ug.mLRAEndIndex = uint32_t(mLRAConstraints.size());
        ug.mRodStretchShearEndIndex = 0;
        ug.mRodBendTwistEndIndex = 0;
        ug.mDihedralBendEndIndex = uint32_t(mDihedralBendConstraints.size());
        ug.mVolumeEndIndex = uint32_t(mVolumeConstraints.size());
        ug.mSkinnedEndIndex = 0;
        mUpdateGroups.push_back(ug);
    }
    mClosestKinematic.clear();
    mClosestKinematic.shrink_to_fit();
}

std::string SoftBodySharedSettings::SaveBinaryState() const {
    static_assert(sizeof(Vertex) == 28 && sizeof(Face) == 16 && sizeof(Edge) == 16 && sizeof(DihedralBend) == 24 &&
                      sizeof(Volume) == 24 && sizeof(LRA) == 12 && sizeof(UpdateGroup) == 28,
                  "binary layout");
    std::string out;
    put_array(out, mVertices);
    put_array(out, mFaces);
    put_array(out, mEdgeConstraints);
    put_array(out, mDihedralBendConstraints);
    put_array(out, mVolumeConstraints);
    uint32_t zero = 0;
    put(out, zero);  // skinned constraints
    put(out, zero);  // skinned constraint normals
    put_array(out, mLRAConstraints);
    put_array(out, mUpdateGroups);
    put(out, zero);  // rod stretch shear
    put(out, zero);  // rod bend twist
    put(out, zero);  // inverse bind matrices
    return out;
}

SoftBodySharedSettings build_settings(const scene::MeshSpec &m) {
    if (!m.skinned.empty()) throw std::runtime_error("skinned settings are built by the reference driver only");
    SoftBodySharedSettings s;
    s.mVertices.resize(m.positions.size());
    for (size_t i = 0; i < m.positions.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            s.mVertices[i].mPosition[k] = m.positions[i][k];
            s.mVertices[i].mVelocity[k] = m.velocities[i][k];
        }
        s.mVertices[i].mInvMass = m.inv_mass[i];
    }
    for (auto &f : m.faces) {
        SoftBodySharedSettings::Face face;
        face.mVertex[0] = f[0];
        face.mVertex[1] = f[1];
        face.mVertex[2] = f[2];
        s.mFaces.push_back(face);
    }
    if (m.create_constraints) {
        s.CreateConstraints(&m.attributes, 1, m.bend_type);
    } else {
        for (size_t i = 0; i < m.edges.size(); ++i) {
            SoftBodySharedSettings::Edge e;
            e.mVertex[0] = m.edges[i][0];
            e.mVertex[1] = m.edges[i][1];
            e.mCompliance = m.edge_compliance[i];
            s.mEdgeConstraints.push_back(e);
        }
        s.CalculateEdgeLengths();
        for (size_t i = 0; i < m.volumes.size(); ++i) {
            SoftBodySharedSettings::Volume v;
            for (int k = 0; k < 4; ++k) v.mVertex[k] = m.volumes[i][k];
            v.mCompliance = m.volume_compliance[i];
            s.mVolumeConstraints.push_back(v);
        }
        s.CalculateVolumeConstraintVolumes();
    }
    s.Optimize();
    if (!m.post_optimize_edge_compliance.empty())
        for (size_t i = 0; i < s.mEdgeConstraints.size() && i < m.post_optimize_edge_compliance.size(); ++i)
            s.mEdgeConstraints[i].mCompliance = m.post_optimize_edge_compliance[i];
    return s;
}

}  // namespace host
}  // namespace jsb
