// Settings parsing and dependency-level scheduling (see schedule.h).

#include "schedule.h"

#include <algorithm>
#include <cstring>

namespace jsb {

namespace {

class ByteReader {
public:
    ByteReader(const uint8_t *p, size_t n) : p_(p), n_(n) {}
    bool u32(uint32_t &v) { return bytes(&v, 4); }
    bool bytes(void *dst, size_t k) {
        if (k > n_ - off_) return false;
        memcpy(dst, p_ + off_, k);
        off_ += k;
        return true;
    }
    template <class T>
    bool array(std::vector<T> &out, size_t elem) {
        uint32_t count;
        if (!u32(count)) return false;
        if (uint64_t(count) * elem > n_ - off_) return false;
        out.resize(count);
        if (count) memcpy(out.data(), p_ + off_, size_t(count) * elem);
        off_ += size_t(count) * elem;
        return true;
    }
    bool skip_array(size_t elem, uint32_t &count) {
        if (!u32(count)) return false;
        if (uint64_t(count) * elem > n_ - off_) return false;
        off_ += size_t(count) * elem;
        return true;
    }
    size_t remaining() const { return n_ - off_; }

private:
    const uint8_t *p_;
    size_t n_, off_ = 0;
};

}  // namespace

std::string parse_settings(const void *blob, size_t len, ParsedSettings &s, bool &unsupported) {
    static_assert(sizeof(ParsedSettings::Vertex) == 28 && sizeof(ParsedSettings::Face) == 16 &&
                      sizeof(ParsedSettings::Edge) == 16 && sizeof(ParsedSettings::Bend) == 24 &&
                      sizeof(ParsedSettings::Volume) == 24 && sizeof(ParsedSettings::LRA) == 12 &&
                      sizeof(ParsedSettings::Group) == 28 && sizeof(ParsedSettings::Skinned) == 52 &&
                      sizeof(ParsedSettings::InvBind) == 68,
                  "SaveBinaryState element sizes");
    unsupported = false;
    if (!blob) return "null settings blob";
    ByteReader r(static_cast<const uint8_t *>(blob), len);
    if (!(r.array(s.vertices, 28) && r.array(s.faces, 16) && r.array(s.edges, 16) && r.array(s.bends, 24) &&
          r.array(s.volumes, 24) && r.array(s.skinned, 52) && r.array(s.skinned_normals, 4) && r.array(s.lras, 12) &&
          r.array(s.groups, 28) && r.skip_array(36, s.num_rod_stretch_shear) && r.skip_array(28, s.num_rod_bend_twist) &&
          r.array(s.inv_binds, 68)))
        return "truncated settings blob";
    s.num_skinned = uint32_t(s.skinned.size());
    s.num_inv_bind = uint32_t(s.inv_binds.size());
    if (r.remaining() != 0) return "trailing bytes after settings blob";
    const uint32_t nv = uint32_t(s.vertices.size());
    if (s.groups.empty()) return "settings have no update groups (SoftBodySharedSettings::Optimize was not called)";
    auto bad = [nv](const uint32_t *v, int k) {
        for (int i = 0; i < k; ++i)
            if (v[i] >= nv) return true;
        return false;
    };
    for (auto &f : s.faces)
        if (bad(f.v, 3)) return "face vertex index out of range";
    for (auto &e : s.edges)
        if (bad(e.v, 2)) return "edge vertex index out of range";
    for (auto &b : s.bends)
        if (bad(b.v, 4)) return "dihedral bend vertex index out of range";
    for (auto &v : s.volumes)
        if (bad(v.v, 4)) return "volume vertex index out of range";
    for (auto &l : s.lras)
        if (bad(l.v, 2)) return "LRA vertex index out of range";
    for (auto &k : s.skinned) {
        if (bad(&k.vertex, 1)) return "skinned constraint vertex index out of range";
        for (auto &w : k.w)
            if (w.weight != 0.0f && w.inv_bind >= s.inv_binds.size()) return "skin weight inverse bind index out of range";
        const uint32_t start = k.normal_info & 0xffffffu, count = k.normal_info >> 24;
        if (uint64_t(start) + count > s.skinned_normals.size()) return "skinned constraint normal range out of range";
    }
    for (uint32_t f : s.skinned_normals)
        if (f >= s.faces.size()) return "skinned constraint normal face index out of range";
    ParsedSettings::Group prev{0, 0, 0, 0, 0, 0, 0};
    for (auto &g : s.groups) {
        if (g.edge < prev.edge || g.lra < prev.lra || g.bend < prev.bend || g.volume < prev.volume || g.rod_ss < prev.rod_ss ||
            g.rod_bt < prev.rod_bt || g.skinned < prev.skinned)
            return "update group end indices decrease";
        prev = g;
    }
    if (prev.edge != s.edges.size() || prev.lra != s.lras.size() || prev.bend != s.bends.size() ||
        prev.volume != s.volumes.size() || prev.rod_ss != s.num_rod_stretch_shear || prev.rod_bt != s.num_rod_bend_twist ||
        prev.skinned != s.num_skinned)
        return "update groups do not cover all constraints";
    if (s.num_rod_stretch_shear || s.num_rod_bend_twist) {
        unsupported = true;
        return "Cosserat rods are not supported by the GPU solver";
    }
    if (s.skinned.size() >= (1u << 24)) {
        unsupported = true;
        return "more than 2^24 skinned constraints";
    }
    if (nv > 65536) {
        unsupported = true;
        return "bodies with more than 65536 vertices are not supported";
    }
    return std::string();
}

Schedule build_schedule(const ParsedSettings &s) {
    const uint32_t nv = uint32_t(s.vertices.size());
    std::vector<int32_t> last_write(nv, -1), last_read(nv, -1);
    struct Item {
        uint32_t level, type, index;
    };
    std::vector<Item> items;
    items.reserve(s.edges.size() + s.bends.size() + s.volumes.size() + s.lras.size() + s.skinned.size());
    uint32_t max_level = 0;
    auto place_rw = [&](const uint32_t *v, int k, uint32_t type, uint32_t index) {
        int32_t lvl = 0;
        for (int i = 0; i < k; ++i) lvl = std::max(lvl, std::max(last_write[v[i]], last_read[v[i]]) + 1);
        for (int i = 0; i < k; ++i) last_write[v[i]] = lvl;
        items.push_back({uint32_t(lvl), type, index});
        max_level = std::max(max_level, uint32_t(lvl));
    };
    ParsedSettings::Group start{0, 0, 0, 0, 0, 0, 0};
    for (size_t g = 0; g < s.groups.size(); ++g) {
        const ParsedSettings::Group &p = g > 0 ? s.groups[g - 1] : start;
        const ParsedSettings::Group &c = s.groups[g];
        for (uint32_t i = p.volume; i < c.volume; ++i) place_rw(s.volumes[i].v, 4, kVolume, i);
        for (uint32_t i = p.bend; i < c.bend; ++i) place_rw(s.bends[i].v, 4, kBend, i);
        for (uint32_t i = p.skinned; i < c.skinned; ++i) place_rw(&s.skinned[i].vertex, 1, kEdge, kSkinRecord | i);
        for (uint32_t i = p.edge; i < c.edge; ++i) place_rw(s.edges[i].v, 2, kEdge, i);
        for (uint32_t i = p.lra; i < c.lra; ++i) {
            uint32_t a = s.lras[i].v[0], b = s.lras[i].v[1];
            int32_t lvl = std::max(last_write[a] + 1, std::max(last_write[b], last_read[b]) + 1);
            if (a == b) lvl = std::max(lvl, last_read[a] + 1);
            last_read[a] = std::max(last_read[a], lvl);
            last_write[b] = lvl;
            items.push_back({uint32_t(lvl), kLRA, i});
            max_level = std::max(max_level, uint32_t(lvl));
        }
    }
    Schedule out;
    const uint32_t n = uint32_t(items.size());
    out.num_records = n;
    out.num_levels = n ? max_level + 1 : 0;
    // counting sort by (level, type), stable in sequence order
    const uint32_t nb = out.num_levels * 4;
    std::vector<uint32_t> count(nb + 1, 0);
    for (const Item &it : items) count[it.level * 4 + it.type + 1]++;
    for (uint32_t k = 0; k < nb; ++k) count[k + 1] += count[k];
    std::vector<uint32_t> bucket_start(count.begin(), count.end());
    std::vector<uint32_t> order(n);
    for (uint32_t k = 0; k < n; ++k) order[count[items[k].level * 4 + items[k].type]++] = k;
    // Inside a level the LRA constraints are ordered by anchor (stably): tethers sharing an anchor sit
    // next to each other, which the adjoint uses to sum their anchor terms in a fixed order. Order
    // inside a level does not change the forward result.
    for (uint32_t l = 0; l < out.num_levels; ++l)
        std::stable_sort(order.begin() + bucket_start[l * 4 + 3], order.begin() + bucket_start[l * 4 + 4],
                         [&](uint32_t a, uint32_t b) { return s.lras[items[a].index].v[0] < s.lras[items[b].index].v[0]; });
    out.levels.resize(size_t(out.num_levels + 2) * 4);
    for (uint32_t l = 0; l < out.num_levels; ++l) {
        out.levels[l * 4 + 0] = bucket_start[l * 4 + 0];
        out.levels[l * 4 + 1] = bucket_start[l * 4 + 1];
        out.levels[l * 4 + 2] = bucket_start[l * 4 + 2];
        out.levels[l * 4 + 3] = bucket_start[l * 4 + 3];
        out.max_level_width = std::max(out.max_level_width, bucket_start[l * 4 + 4] - bucket_start[l * 4]);
    }
    for (uint32_t l = out.num_levels; l < out.num_levels + 2; ++l)
        for (int k = 0; k < 4; ++k) out.levels[l * 4 + k] = n;
    out.records.resize(size_t(n) * 4);
    out.source.resize(n);
    auto fbits = [](float f) {
        uint32_t u;
        memcpy(&u, &f, 4);
        return u;
    };
    for (uint32_t k = 0; k < n; ++k) {
        const Item &it = items[order[k]];
        uint32_t *r = &out.records[size_t(k) * 4];
        switch (it.type) {
            case kBend: {
                const auto &b = s.bends[it.index];
                r[0] = b.v[0] | (b.v[1] << 16);
                r[1] = b.v[2] | (b.v[3] << 16);
                r[2] = fbits(b.compliance);
                r[3] = fbits(b.initial_angle);
                break;
            }
            case kVolume: {
                const auto &v = s.volumes[it.index];
                r[0] = v.v[0] | (v.v[1] << 16);
                r[1] = v.v[2] | (v.v[3] << 16);
                r[2] = fbits(v.six_rest_volume);
                r[3] = fbits(v.compliance);
                break;
            }
            case kEdge: {
                if (it.index & kSkinRecord) {
                    r[0] = s.skinned[it.index & ~kSkinRecord].vertex;
                    r[1] = it.index;
                    r[2] = 0;
                    r[3] = 0;
                    break;
                }
                const auto &e = s.edges[it.index];
                r[0] = e.v[0] | (e.v[1] << 16);
                r[1] = 0;
                r[2] = fbits(e.rest);
                r[3] = fbits(e.compliance);
                break;
            }
            default: {
                const auto &l = s.lras[it.index];
                r[0] = l.v[0] | (l.v[1] << 16);
                r[1] = 0;
                r[2] = fbits(l.max_distance);
                r[3] = 0;
                break;
            }
        }
        out.source[k] = (it.index & kSkinRecord) ? ((kSkinSource << 28) | (it.index & ~kSkinRecord)) : ((it.type << 28) | it.index);
    }
    // padded device layout
    auto pad = [](uint32_t v) { return (v + 31u) & ~31u; };
    out.padded_levels.resize(size_t(out.num_levels + 2) * 4);
    uint32_t slot = 0;
    for (uint32_t l = 0; l < out.num_levels; ++l) {
        const uint32_t *lv = &out.levels[l * 4];
        const uint32_t next = out.levels[(l + 1) * 4];
        uint32_t nb = lv[1] - lv[0], nvol = lv[2] - lv[1], ne = lv[3] - lv[2], nl = next - lv[3];
        uint32_t b_end = pad(nb), v_end = b_end + pad(nvol), e_end = v_end + pad(ne), total = e_end + pad(nl);
        out.padded_levels[l * 4 + 0] = slot;
        out.padded_levels[l * 4 + 1] = b_end;
        out.padded_levels[l * 4 + 2] = v_end;
        out.padded_levels[l * 4 + 3] = e_end;
        out.max_level_slots = std::max(out.max_level_slots, total);
        slot += total;
    }
    out.num_slots = slot;
    for (uint32_t l = out.num_levels; l < out.num_levels + 2; ++l) {
        out.padded_levels[l * 4 + 0] = slot;
        out.padded_levels[l * 4 + 1] = out.padded_levels[l * 4 + 2] = out.padded_levels[l * 4 + 3] = 0;
    }
    out.padded_records.assign(size_t(slot) * 4, 0);
    out.padded_source.assign(slot, 0xffffffffu);
    for (uint32_t k = 0; k < slot; ++k) out.padded_records[size_t(k) * 4] = kPadRecord;
    for (uint32_t l = 0; l < out.num_levels; ++l) {
        const uint32_t *lv = &out.levels[l * 4];
        const uint32_t next = out.levels[(l + 1) * 4];
        const uint32_t base = out.padded_levels[l * 4];
        const uint32_t group_first[4] = {lv[0], lv[1], lv[2], lv[3]};
        const uint32_t group_last[4] = {lv[1], lv[2], lv[3], next};
        const uint32_t group_slot[4] = {0, out.padded_levels[l * 4 + 1], out.padded_levels[l * 4 + 2], out.padded_levels[l * 4 + 3]};
        for (int t = 0; t < 4; ++t)
            for (uint32_t c = group_first[t]; c < group_last[t]; ++c) {
                uint32_t dst = base + group_slot[t] + (c - group_first[t]);
                for (int k = 0; k < 4; ++k) out.padded_records[size_t(dst) * 4 + k] = out.records[size_t(c) * 4 + k];
                out.padded_source[dst] = out.source[c];
            }
    }
    return out;
}

bool build_step_schedule(const ParsedSettings &s, uint32_t num_iterations, StepSchedule &out, bool with_source) {
    out = StepSchedule();
    if (num_iterations < 2) return false;
    const uint32_t nv = uint32_t(s.vertices.size());
    std::vector<int32_t> last_write(nv, -1), last_read(nv, -1);
    struct Item {
        uint32_t level, type, index, substep;
    };
    std::vector<Item> items;
    uint32_t cur_substep = 0;
    const size_t per_substep = s.edges.size() + s.bends.size() + s.volumes.size() + s.lras.size() + s.skinned.size() + nv;
    items.reserve(per_substep * num_iterations);
    uint32_t max_level = 0;
    auto place_rw = [&](const uint32_t *v, int k, uint32_t type, uint32_t index) {
        int32_t lvl = 0;
        for (int i = 0; i < k; ++i) lvl = std::max(lvl, std::max(last_write[v[i]], last_read[v[i]]) + 1);
        for (int i = 0; i < k; ++i) last_write[v[i]] = lvl;
        items.push_back({uint32_t(lvl), type, index, cur_substep});
        max_level = std::max(max_level, uint32_t(lvl));
    };
    for (uint32_t it = 0; it < num_iterations; ++it) {
        cur_substep = it;
        if (it > 0)
            for (uint32_t v = 0; v < nv; ++v) place_rw(&v, 1, kVertexOp, v);
        ParsedSettings::Group start{0, 0, 0, 0, 0, 0, 0};
        for (size_t g = 0; g < s.groups.size(); ++g) {
            const ParsedSettings::Group &p = g > 0 ? s.groups[g - 1] : start;
            const ParsedSettings::Group &c = s.groups[g];
            for (uint32_t i = p.volume; i < c.volume; ++i) place_rw(s.volumes[i].v, 4, kVolume, i);
            for (uint32_t i = p.bend; i < c.bend; ++i) place_rw(s.bends[i].v, 4, kBend, i);
            for (uint32_t i = p.skinned; i < c.skinned; ++i) place_rw(&s.skinned[i].vertex, 1, kEdge, kSkinRecord | i);
            for (uint32_t i = p.edge; i < c.edge; ++i) place_rw(s.edges[i].v, 2, kEdge, i);
            for (uint32_t i = p.lra; i < c.lra; ++i) {
                uint32_t a = s.lras[i].v[0], b = s.lras[i].v[1];
                int32_t lvl = std::max(last_write[a] + 1, std::max(last_write[b], last_read[b]) + 1);
                if (a == b) lvl = std::max(lvl, last_read[a] + 1);
                last_read[a] = std::max(last_read[a], lvl);
                last_write[b] = lvl;
                items.push_back({uint32_t(lvl), kLRA, i, it});
                max_level = std::max(max_level, uint32_t(lvl));
            }
        }
    }
    if (items.empty()) return false;
    const uint32_t L = max_level + 1;
    // per (level, type) counts, padded to multiples of 32 slots
    std::vector<uint32_t> count(size_t(L) * 5, 0);
    for (const Item &it : items) count[size_t(it.level) * 5 + it.type]++;
    auto pad = [](uint32_t v) { return (v + 31u) & ~31u; };
    std::vector<uint32_t> slot_of(size_t(L) * 5);  // next free slot of each (level, type)
    out.levels.resize(size_t(L) * 4);
    uint32_t slot = 0;
    for (uint32_t l = 0; l < L; ++l) {
        const uint32_t *c = &count[size_t(l) * 5];
        const uint32_t be = pad(c[kBend]), ve = be + pad(c[kVolume]), ee = ve + pad(c[kEdge]), le = ee + pad(c[kLRA]);
        const uint32_t total = le + pad(c[kVertexOp]);
        if (total >= 65536u) {
            out = StepSchedule();
            return false;
        }
        out.levels[l * 4 + 0] = slot;
        out.levels[l * 4 + 1] = be | (ve << 16);
        out.levels[l * 4 + 2] = ee | (le << 16);
        out.levels[l * 4 + 3] = total;
        slot_of[size_t(l) * 5 + kBend] = slot;
        slot_of[size_t(l) * 5 + kVolume] = slot + be;
        slot_of[size_t(l) * 5 + kEdge] = slot + ve;
        slot_of[size_t(l) * 5 + kLRA] = slot + ee;
        slot_of[size_t(l) * 5 + kVertexOp] = slot + le;
        out.max_level_slots = std::max(out.max_level_slots, total);
        slot += total;
    }
    out.num_levels = L;
    out.num_slots = slot;
    out.num_iterations = num_iterations;
    out.records.assign(size_t(slot) * 4, 0);
    for (uint32_t k = 0; k < slot; ++k) out.records[size_t(k) * 4] = kPadRecord;
    if (with_source) out.source.assign(size_t(slot) * 2, 0xffffffffu);
    auto fbits = [](float f) {
        uint32_t u;
        memcpy(&u, &f, 4);
        return u;
    };
    // items are in sequence order, so filling each (level, type) in that order keeps the in-level order
    // of build_schedule (LRA constraints are reordered by anchor below, as there)
    for (const Item &it : items) {
        const uint32_t k = slot_of[size_t(it.level) * 5 + it.type]++;
        uint32_t *r = &out.records[size_t(k) * 4];
        if (with_source) {
            out.source[size_t(k) * 2] =
                (it.index & kSkinRecord) ? ((kSkinSource << 28) | (it.index & ~kSkinRecord)) : ((it.type << 28) | it.index);
            out.source[size_t(k) * 2 + 1] = it.substep;
        }
        switch (it.type) {
            case kBend: {
                const auto &b = s.bends[it.index];
                r[0] = b.v[0] | (b.v[1] << 16);
                r[1] = b.v[2] | (b.v[3] << 16);
                r[2] = fbits(b.compliance);
                r[3] = fbits(b.initial_angle);
                break;
            }
            case kVolume: {
                const auto &v = s.volumes[it.index];
                r[0] = v.v[0] | (v.v[1] << 16);
                r[1] = v.v[2] | (v.v[3] << 16);
                r[2] = fbits(v.six_rest_volume);
                r[3] = fbits(v.compliance);
                break;
            }
            case kEdge: {
                if (it.index & kSkinRecord) {
                    r[0] = s.skinned[it.index & ~kSkinRecord].vertex | (it.substep << 16);
                    r[1] = it.index;
                    break;
                }
                const auto &e = s.edges[it.index];
                r[0] = e.v[0] | (e.v[1] << 16);
                r[2] = fbits(e.rest);
                r[3] = fbits(e.compliance);
                break;
            }
            case kLRA: {
                const auto &l = s.lras[it.index];
                r[0] = l.v[0] | (l.v[1] << 16);
                r[2] = fbits(l.max_distance);
                break;
            }
            default:
                r[0] = it.index;
                r[1] = it.substep;
                break;
        }
    }
    // LRA constraints of a level ordered by anchor (stably; the slots before the padding)
    for (uint32_t l = 0; l < L; ++l) {
        const uint32_t first = out.levels[l * 4] + (out.levels[l * 4 + 2] & 0xffffu);
        const uint32_t n = count[size_t(l) * 5 + kLRA];
        if (n < 2) continue;
        std::vector<uint32_t> idx(n);
        for (uint32_t k = 0; k < n; ++k) idx[k] = k;
        std::stable_sort(idx.begin(), idx.end(), [&](uint32_t a, uint32_t b) {
            return (out.records[size_t(first + a) * 4] & 0xffffu) < (out.records[size_t(first + b) * 4] & 0xffffu);
        });
        std::vector<uint32_t> rec(size_t(n) * 4), src;
        for (uint32_t k = 0; k < n; ++k)
            for (int w = 0; w < 4; ++w) rec[size_t(k) * 4 + w] = out.records[size_t(first + idx[k]) * 4 + w];
        std::copy(rec.begin(), rec.end(), out.records.begin() + size_t(first) * 4);
        if (with_source) {
            src.resize(size_t(n) * 2);
            for (uint32_t k = 0; k < n; ++k)
                for (int w = 0; w < 2; ++w) src[size_t(k) * 2 + w] = out.source[size_t(first + idx[k]) * 2 + w];
            std::copy(src.begin(), src.end(), out.source.begin() + size_t(first) * 2);
        }
    }
    return true;
}

namespace {

// First-fit colours of a sequence of constraints over vertex sets: per vertex the colours in which it
// is written (w) and read (r), as bit masks grown on demand.
class Colouring {
public:
    explicit Colouring(uint32_t nv) : nv_(nv), words_(1), w_(nv, 0), r_(nv, 0) {}
    // Smallest colour in which none of `writes` is written or read and none of `reads` is written.
    uint32_t place(const uint32_t *writes, int nw, const uint32_t *reads, int nr) {
        for (uint32_t word = 0;; ++word) {
            if (word == words_) grow();
            uint64_t used = 0;
            for (int i = 0; i < nw; ++i) used |= w_[size_t(writes[i]) * words_ + word] | r_[size_t(writes[i]) * words_ + word];
            for (int i = 0; i < nr; ++i) used |= w_[size_t(reads[i]) * words_ + word];
            if (used != ~uint64_t(0)) {
                const uint32_t bit = uint32_t(__builtin_ctzll(~used));
                for (int i = 0; i < nw; ++i) w_[size_t(writes[i]) * words_ + word] |= uint64_t(1) << bit;
                for (int i = 0; i < nr; ++i) r_[size_t(reads[i]) * words_ + word] |= uint64_t(1) << bit;
                return word * 64 + bit;
            }
        }
    }

private:
    void grow() {
        const uint32_t nw = words_ * 2;
        std::vector<uint64_t> w(size_t(nv_) * nw, 0), r(size_t(nv_) * nw, 0);
        for (uint32_t v = 0; v < nv_; ++v)
            for (uint32_t k = 0; k < words_; ++k) {
                w[size_t(v) * nw + k] = w_[size_t(v) * words_ + k];
                r[size_t(v) * nw + k] = r_[size_t(v) * words_ + k];
            }
        w_.swap(w);
        r_.swap(r);
        words_ = nw;
    }
    uint32_t nv_, words_;
    std::vector<uint64_t> w_, r_;
};

// Indices 0..n-1 ordered by colour, stably.
std::vector<uint32_t> by_colour(const std::vector<uint32_t> &colour) {
    std::vector<uint32_t> order(colour.size());
    for (uint32_t i = 0; i < order.size(); ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return colour[a] < colour[b]; });
    return order;
}

template <class T>
void put_array(std::vector<uint8_t> &out, const std::vector<T> &items, const std::vector<uint32_t> *order) {
    const uint32_t n = uint32_t(items.size());
    const uint8_t *pn = reinterpret_cast<const uint8_t *>(&n);
    out.insert(out.end(), pn, pn + 4);
    for (uint32_t k = 0; k < n; ++k) {
        const uint8_t *p = reinterpret_cast<const uint8_t *>(&items[order ? (*order)[k] : k]);
        out.insert(out.end(), p, p + sizeof(T));
    }
}

}  // namespace

std::vector<uint8_t> regroup_settings(const ParsedSettings &s, std::vector<uint32_t> &remap) {
    remap.clear();
    if (!s.skinned.empty()) return {};  // (not regrouped: the caller reports it)
    const uint32_t nv = uint32_t(s.vertices.size());
    std::vector<uint32_t> cv(s.volumes.size()), cb(s.bends.size()), ce(s.edges.size()), cl(s.lras.size());
    {
        Colouring c(nv);
        for (size_t i = 0; i < s.volumes.size(); ++i) cv[i] = c.place(s.volumes[i].v, 4, nullptr, 0);
    }
    {
        Colouring c(nv);
        for (size_t i = 0; i < s.bends.size(); ++i) cb[i] = c.place(s.bends[i].v, 4, nullptr, 0);
    }
    {
        Colouring c(nv);
        for (size_t i = 0; i < s.edges.size(); ++i) ce[i] = c.place(s.edges[i].v, 2, nullptr, 0);
    }
    {
        Colouring c(nv);
        for (size_t i = 0; i < s.lras.size(); ++i) {
            const uint32_t a = s.lras[i].v[0], b = s.lras[i].v[1];
            cl[i] = a == b ? c.place(&b, 1, nullptr, 0) : c.place(&b, 1, &a, 1);
        }
    }
    // The reference's sequence of one group is its volumes, bends, edges, LRA; colour the constraints of
    // each type in the order they came (parallel groups first, the non-parallel group last).
    const std::vector<uint32_t> ov = by_colour(cv), ob = by_colour(cb), oe = by_colour(ce), ol = by_colour(cl);
    remap.clear();
    remap.insert(remap.end(), oe.begin(), oe.end());
    remap.insert(remap.end(), ob.begin(), ob.end());
    remap.insert(remap.end(), ov.begin(), ov.end());
    remap.insert(remap.end(), ol.begin(), ol.end());
    std::vector<uint8_t> out;
    put_array(out, s.vertices, nullptr);
    put_array(out, s.faces, nullptr);
    put_array(out, s.edges, &oe);
    put_array(out, s.bends, &ob);
    put_array(out, s.volumes, &ov);
    const std::vector<uint32_t> none;
    put_array(out, none, nullptr);  // skinned constraints
    put_array(out, none, nullptr);  // skinned constraint normals
    put_array(out, s.lras, &ol);
    ParsedSettings::Group g{uint32_t(s.edges.size()), uint32_t(s.lras.size()), 0, 0, uint32_t(s.bends.size()),
                            uint32_t(s.volumes.size()), 0};
    put_array(out, std::vector<ParsedSettings::Group>{g}, nullptr);
    put_array(out, none, nullptr);  // rod stretch-shear
    put_array(out, none, nullptr);  // rod bend-twist
    put_array(out, none, nullptr);  // inverse bind matrices
    return out;
}

std::vector<uint32_t> build_stage_chunks(const std::vector<uint32_t> &levels4, uint32_t num_levels, bool per_substep,
                                         uint32_t half_slots) {
    std::vector<uint32_t> out;
    auto slots = [&](uint32_t l) { return per_substep ? levels4[(l + 1) * 4] - levels4[l * 4] : levels4[l * 4 + 3]; };
    uint32_t l = 0;
    while (l < num_levels) {
        const uint32_t first = levels4[l * 4];
        uint32_t end = l, total = 0;
        while (end < num_levels && end - l < kStageLevels && total + slots(end) <= half_slots) total += slots(end++);
        if (end == l) {  // one level wider than a half: stage its first half_slots slots
            end = l + 1;
            total = half_slots;
        }
        out.insert(out.end(), {l, end, first, total});
        l = end;
    }
    return out;
}

}  // namespace jsb
