// ps_circuit.cpp -- compiled circuits: plain (one launch per op) and fused
// (segments of gates applied in one tableau pass + measurement phases), with
// optional CUDA-graph capture.  Replaces the reference's op-by-op driver
// CliffordCircuit::Execute (CliffordCircuit.hpp:131-135).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <deque>
#include <memory>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "../../include/plaquette_gpu.h"
#include "ps_frame.h"
#include "ps_frame_dev.h"
#include "ps_internal.h"
#include "ps_segment.cuh"

namespace ps {

namespace {

// Detector d, word k: XOR of the records idx[off[d] .. off[d+1]) (coalesced
// over words).
__global__ void detector_kernel(const u64 *__restrict__ res, int64_t w, const uint32_t *__restrict__ idx,
                                const uint64_t *__restrict__ off, int64_t ndet, u64 *__restrict__ out) {
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < ndet * w;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t d = e / w, k = e - d * w;
        u64 v = 0ull;
        for (uint64_t j = off[d]; j < off[d + 1]; ++j) v ^= res[(int64_t)idx[j] * w + k];
        out[e] = v;
    }
}

__global__ void set_params_kernel(RunParams *p, uint64_t seed, uint64_t event_base, uint64_t word_base) {
    p->seed = seed;
    p->event_base = event_base;
    p->word_base = word_base;
    p->pad = 0;
}

enum StepKind { K_GATE, K_CHANNEL, K_MEAS, K_SEGMENT, K_INIT };

struct Step {
    StepKind kind;
    int32_t code = 0;
    int64_t a = 0, b = 0;
    int32_t rec = -1;       // K_GATE: flag record (circuit-local)
    int32_t count = 0;      // K_CHANNEL: 3 / 15; K_MEAS: number of ops
    int32_t first = 0;      // K_MEAS: first MeasOp; K_SEGMENT: segment index; K_CHANNEL: thr offset
    uint32_t event = 0;     // K_CHANNEL event offset
    int32_t table = 0;      // K_CHANNEL: its channel table (survival products, estimate factors)
};

struct SegHost {
    std::vector<SegLayer> layers;
    std::vector<SegRun> runs;
    std::vector<SegGate> gates;
    std::vector<SegSign> signs;
    std::vector<int32_t> cols;
    std::vector<NoiseSlot> slots;
    std::vector<int32_t> slot_op;     // op index of each slot
    size_t op0 = 0, op1 = 0;          // the segment's ops [op0, op1)
    std::vector<int32_t> recsig_rec;  // record of each reset-X slot
    // resident form (res_slots > 0)
    int32_t res_slots = 0;
    std::vector<uint16_t> res_cols;   // [RC][32]
    std::vector<ResOp> res_ops;       // [nlayers][RC][32]
    std::vector<uint32_t> prop_desc;  // [4 nslots + nsigns]
    std::vector<uint32_t> prop_sup;
    SegmentDev dev{};
    void *dev_block = nullptr;
};

// Device copy of a host table, owned by the circuit.  The copy is ordered on
// the state's stream (pageable source: staged before the call returns).
template <class T> int upload(ps_state *h, std::vector<void *> &owned, const std::vector<T> &v, T **out) {
    *out = nullptr;
    if (v.empty()) return OK;
    void *p = nullptr;
    if (dev_alloc(h, &p, v.size() * sizeof(T)) != OK) return E_NOMEM;
    owned.push_back(p);
    PS_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    *out = static_cast<T *>(p);
    return OK;
}

// ---- compile cache ------------------------------------------------------
// The host-side products of compiling one circuit -- the plan's steps, the
// fused segments' schedules, the measurement list and the shared-x/z sign
// program -- depend on the qubit count, the options, whether the state is a
// valid tableau, and the op and parameter tables, but not on the shots, the
// seed or any device memory.  They are kept per process (the most recent
// kPlanCacheMax), so that compiling a circuit again (a served or batched
// job of a shape seen before) only allocates, uploads and captures.
struct PlanCacheEntry {
    std::vector<Step> steps;
    std::vector<SegHost> segs;      // host fields only (no device pointers)
    std::vector<MeasOp> meas;       // without record or forced pointers
    std::vector<int32_t> meas_op;
    bool has_frame = false;
    FrameProgram fprog;
};
constexpr size_t kPlanCacheMax = 128;
std::mutex g_plan_mu;
std::map<std::string, std::shared_ptr<const PlanCacheEntry>> g_plan;
std::deque<std::string> g_plan_order;  // insertion order, oldest first
uint64_t g_plan_hits = 0, g_plan_misses = 0;

std::string plan_key(const ps_state *h, const ps_circuit_options &o, const std::vector<ps_op> &ops, const float *params,
                     uint64_t nparams) {
    std::string k;
    auto put = [&](const void *p, size_t n) { k.append(static_cast<const char *>(p), n); };
    const int64_t n = h->n;
    const int32_t valid = h->valid ? 1 : 0;
    const uint64_t nops = ops.size();
    put(&n, sizeof n);
    put(&valid, sizeof valid);
    put(&o, sizeof o);
    put(&nops, sizeof nops);
    if (nops) put(ops.data(), nops * sizeof(ps_op));
    put(&nparams, sizeof nparams);
    if (nparams) put(params, nparams * sizeof(float));
    return k;
}

std::shared_ptr<const PlanCacheEntry> plan_lookup(const std::string &key) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plan.find(key);
    if (it == g_plan.end()) {
        ++g_plan_misses;
        return nullptr;
    }
    ++g_plan_hits;
    return it->second;
}

void plan_store(const std::string &key, std::shared_ptr<const PlanCacheEntry> e) {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (g_plan.count(key)) return;
    g_plan[key] = std::move(e);
    g_plan_order.push_back(key);
    while (g_plan_order.size() > kPlanCacheMax) {
        g_plan.erase(g_plan_order.front());
        g_plan_order.pop_front();
    }
}

}  // namespace

}  // namespace ps

using namespace ps;

struct ps_circuit {
    ps_state *h = nullptr;
    ps_circuit_options opts{};
    ps_circuit_stats stats{};
    std::vector<Step> steps;
    std::vector<MeasOp> meas;       // host copy
    MeasOp *d_meas = nullptr;
    RunParams *d_params = nullptr;
    uint64_t *d_thr = nullptr;
    std::vector<uint64_t> thr_host; // the distinct channel tables (host copy of d_thr)
    uint32_t *d_psurv = nullptr;    // plain form: survival products of each distinct table, 64 words each
    std::vector<ChannelEst> pest;   // plain form: estimate factors of each distinct table
    u64 **d_recs = nullptr;
    u64 *d_masks = nullptr;         // plain-mode channel masks (4w)
    u64 *d_forced = nullptr;        // [nm][w]
    NoiseEntry *d_entries = nullptr;
    u64 *d_dense = nullptr;
    int32_t *d_entry_count = nullptr;
    int32_t entry_cap = 0;
    std::vector<SegHost> segs;
    std::vector<void *> owned;
    std::vector<int64_t> rec_ids;   // state record ids of the circuit's M/R
    u64 *d_res_block = nullptr;     // [nm][w] (owned by the state)
    u64 *d_det_block = nullptr;
    uint64_t num_events = 0;
    std::vector<int32_t> meas_op;   // op index of each MeasOp
    // Shared-x/z plan of runs from |0...0> (ps_frame.h), when the circuit
    // has no per-shot conditional gates.
    bool frame_ok = false;
    bool force_per_shot = false;    // measurement statistics need the per-shot plan
    // The per-shot plan's device schedules (ensure_segments_dev): -1 not
    // built yet, else the status of the one attempt.
    int seg_dev_status = -1;
    bool seg_dev_ready = false;
    size_t max_slots = 0;           // channels of the largest segment
    FrameProgram fprog;
    FrameOp *d_fops = nullptr;
    uint32_t *d_ftab = nullptr;
    int32_t *d_frand = nullptr;
    uint64_t *d_fxz = nullptr;
    // The shared-x/z plan as a job table of one job (ps_frame_dev.h): one
    // sign-kernel launch and one x / z broadcast beside it on a side stream.
    FrameTable ftable;
    int32_t *d_ferr = nullptr;       // the sign kernel's error word (a bounded wait gave up)
    FrameJobDev fjob{};              // host copies of the one-job table's entries (batches gather them)
    BroadcastJobDev fbjob{};
    cudaStream_t fstream = nullptr;  // the broadcast's side stream
    cudaEvent_t fev[2] = {nullptr, nullptr};
    // ps_circuit_copy_records_async: the copy stream (own or the caller's),
    // the end of the run it copies, the end of the copy, and the error word
    // in pinned host memory.
    cudaStream_t cstream_own = nullptr;
    cudaEvent_t ev_ran = nullptr, ev_copied = nullptr;
    bool copy_pending = false;
    int32_t *h_err = nullptr;
    cudaGraph_t graph[2] = {nullptr, nullptr};      // [reset_state]
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
};

namespace ps {
namespace {

bool is_gate(int32_t c) { return c == OP_H || c == OP_S || c == OP_CX || c == OP_CZ || c == OP_H_IF || c == OP_S_IF; }
bool is_sign(int32_t c) { return c == OP_X || c == OP_Y || c == OP_Z; }
bool is_meas(int32_t c) { return c == OP_M || c == OP_R; }
bool is_channel(int32_t c) { return c == OP_PAULI1 || c == OP_PAULI2; }

// The dummy column of residue r (kSegDummyCols zero columns follow the nq
// columns of every tile row, one per bank group): a pad lane of a gate group
// touches the dummy of a residue no other lane of its group uses.
inline uint16_t dummy_col(int nq, int r) { return (uint16_t)(nq + ((r - nq) % 8 + 8) % 8); }

// Lane groups needed by a run of gates of one code: a 16-byte shared-memory
// access is served 8 lanes at a time (8 cells x 16 B = one 128-byte bank
// row), so every group of 8 lanes needs distinct residues mod 8 -- the bank
// group of a tile cell -- on a and, for two-qubit gates, on b.  Gates are the
// edges of a bipartite multigraph on 8 + 8 residues and a group is a matching,
// so the fewest groups is the largest residue degree (Koenig's edge-colouring
// theorem).
int lane_groups_needed(const std::vector<SegGate> &gs, bool two) {
    int da[8] = {0, 0, 0, 0, 0, 0, 0, 0}, db[8] = {0, 0, 0, 0, 0, 0, 0, 0}, D = 0;
    for (const SegGate &g : gs) {
        D = std::max(D, ++da[g.a & 7]);
        if (two) D = std::max(D, ++db[g.b & 7]);
    }
    return D;
}

// Splits gates (all of one code) into exactly that many groups of 8 lanes:
// the residue multigraph is padded with dummy edges to a D-regular one, whose
// D perfect matchings (Kuhn's augmenting paths; Hall's condition holds in a
// regular bipartite multigraph) are the groups.  Dummy edges become pad lanes
// on the dummy columns of their residues.
std::vector<std::vector<SegGate>> lane_groups(const std::vector<SegGate> &gs, bool two, int nq, int32_t code) {
    std::vector<SegGate> m[8][8];
    int dm[8][8] = {}, da[8] = {}, db[8] = {};
    for (const SegGate &g : gs) {
        const int a = g.a & 7, b = two ? (g.b & 7) : a;
        m[a][b].push_back(g);
        da[a]++;
        db[b]++;
    }
    const int D = lane_groups_needed(gs, two);
    if (!two) {
        for (int r = 0; r < 8; ++r) dm[r][r] = D - da[r];
    } else {
        for (int a = 0; a < 8; ++a)
            while (da[a] < D) {
                int best = -1;
                for (int b = 0; b < 8; ++b)
                    if (db[b] < D && (best < 0 || db[b] < db[best])) best = b;
                dm[a][best]++;
                da[a]++;
                db[best]++;
            }
    }
    std::vector<std::vector<SegGate>> out;
    for (int k = 0; k < D; ++k) {
        int match_b[8];
        for (int b = 0; b < 8; ++b) match_b[b] = -1;
        std::function<bool(int, bool *)> try_a = [&](int a, bool *seen) -> bool {
            for (int b = 0; b < 8; ++b)
                if ((!m[a][b].empty() || dm[a][b] > 0) && !seen[b]) {
                    seen[b] = true;
                    if (match_b[b] < 0 || try_a(match_b[b], seen)) {
                        match_b[b] = a;
                        return true;
                    }
                }
            return false;
        };
        for (int a = 0; a < 8; ++a) {
            bool seen[8] = {false, false, false, false, false, false, false, false};
            try_a(a, seen);
        }
        std::vector<SegGate> grp;
        for (int b = 0; b < 8; ++b) {
            const int a = match_b[b];
            if (a < 0) continue;  // unreachable for a regular multigraph
            if (!m[a][b].empty()) {
                grp.push_back(m[a][b].back());
                m[a][b].pop_back();
            } else {
                dm[a][b]--;
                grp.push_back(SegGate{dummy_col(nq, a), dummy_col(nq, two ? b : a), code});
            }
        }
        out.push_back(std::move(grp));
    }
    return out;
}

// Builds the layered schedule of one segment.  Gates go to the first layer
// after the last use of their qubits; sign ops (Pauli gates, channel
// outcomes, reset X) are applied after the gates of the layer where their
// qubits were last touched, which keeps every op's order relative to the
// gates on its own qubits.
int build_segment(ps_circuit *c, const std::vector<ps_op> &ops, size_t i0, size_t i1,
                  const std::vector<uint32_t> &event_of, const std::vector<int32_t> &rec_of,
                  const std::vector<int32_t> &thr_off, const std::vector<std::pair<int64_t, int32_t>> &pre_signs,
                  SegHost &seg) {
    seg.op0 = i0;
    seg.op1 = i1;
    std::set<int32_t> qset;
    for (auto &ps_ : pre_signs) qset.insert((int32_t)ps_.first);
    for (size_t i = i0; i < i1; ++i) {
        qset.insert(ops[i].a);
        if (ops[i].code == OP_CX || ops[i].code == OP_CZ || ops[i].code == OP_PAULI2) qset.insert(ops[i].b);
    }
    seg.cols.assign(qset.begin(), qset.end());
    std::map<int32_t, int32_t> loc;
    for (size_t l = 0; l < seg.cols.size(); ++l) loc[seg.cols[l]] = (int32_t)l;

    struct LayerBuild {
        std::vector<SegGate> gates;
        std::vector<SegSign> signs;
        std::vector<NoiseSlot> slots;
        std::vector<int32_t> slot_ops;
    };
    std::vector<LayerBuild> L(1);  // layer 0: no gates (signs before any gate)
    std::map<int32_t, int32_t> last;  // local col -> layer of last touch
    auto lastof = [&](int32_t q) { auto it = last.find(q); return it == last.end() ? 0 : it->second; };
    auto ensure = [&](int32_t layer) { while ((int32_t)L.size() <= layer) L.emplace_back(); };

    for (auto &pr : pre_signs) {
        SegSign s{(uint16_t)loc[(int32_t)pr.first], (uint16_t)SIGN_REC_X, (int32_t)seg.recsig_rec.size()};
        seg.recsig_rec.push_back(pr.second);
        L[0].signs.push_back(s);
    }
    for (size_t i = i0; i < i1; ++i) {
        const ps_op &o = ops[i];
        const int32_t a = loc[o.a];
        if (is_gate(o.code)) {
            int32_t layer;
            SegGate g{(uint16_t)a, 0, o.code};
            if (o.code == OP_CX || o.code == OP_CZ) {
                const int32_t b = loc[o.b];
                layer = std::max(lastof(a), lastof(b)) + 1;
                g.b = (uint16_t)b;
                last[a] = last[b] = layer;
            } else {
                layer = lastof(a) + 1;
                last[a] = layer;
                if (o.code == OP_H_IF || o.code == OP_S_IF) g.code_rec = o.code | (o.c << 4);
            }
            ensure(layer);
            L[layer].gates.push_back(g);
        } else if (is_sign(o.code)) {
            const int32_t layer = lastof(a);
            SegSign s{(uint16_t)a, (uint16_t)(o.code == OP_X ? SIGN_X : o.code == OP_Y ? SIGN_Y : SIGN_Z), -1};
            L[layer].signs.push_back(s);
        } else if (is_channel(o.code)) {
            NoiseSlot sl{};
            sl.a = a;
            sl.b = o.code == OP_PAULI2 ? loc[o.b] : -1;
            int32_t layer = lastof(a);
            if (sl.b >= 0) {
                layer = std::max(layer, lastof(sl.b));
                last[sl.b] = layer;
            }
            last[a] = layer;
            sl.layer = layer;
            sl.count = o.code == OP_PAULI2 ? 15 : 3;
            sl.thr_off = thr_off[i];
            sl.event = event_of[i];
            L[layer].slots.push_back(sl);
            L[layer].slot_ops.push_back((int32_t)i);
        }
    }
    const int nq = (int)seg.cols.size();
    const int nl = (int)L.size();

    // ---- resident form: columns kept in registers by their owner lane.
    // Eligible without per-shot conditional gates (their effect on a Pauli
    // would depend on the shot).  The resident set is independent in the
    // segment's two-qubit-gate graph: on a bipartite graph (data / ancilla)
    // the side with more gate touches, else greedily by touches.
    std::vector<std::vector<SegGate>> all_gates(nl);
    for (int l = 0; l < nl; ++l) all_gates[l] = L[l].gates;
    bool res_form = c->opts.seg_resident == 1;
    std::vector<int> touches(nq, 0);
    std::vector<std::vector<int>> adj(nq);
    for (int l = 0; l < nl && res_form; ++l)
        for (const SegGate &g : L[l].gates) {
            const int32_t code = g.code_rec & 15;
            if (code == OP_H_IF || code == OP_S_IF) res_form = false;
            touches[g.a]++;
            if (code == OP_CX || code == OP_CZ) {
                touches[g.b]++;
                adj[g.a].push_back(g.b);
                adj[g.b].push_back(g.a);
            }
        }
    std::vector<int> resident;  // local columns
    if (res_form) {
        std::vector<int> color(nq, -1);
        std::vector<char> pick(nq, 0);
        for (int s0 = 0; s0 < nq; ++s0) {
            if (color[s0] >= 0 || touches[s0] == 0) continue;
            std::vector<int> comp{s0};
            color[s0] = 0;
            bool bip = true;
            for (size_t h = 0; h < comp.size(); ++h)
                for (int v : adj[comp[h]]) {
                    if (color[v] < 0) {
                        color[v] = 1 - color[comp[h]];
                        comp.push_back(v);
                    } else if (color[v] == color[comp[h]]) {
                        bip = false;
                    }
                }
            if (bip) {
                long t0 = 0, t1 = 0;
                for (int v : comp) (color[v] ? t1 : t0) += touches[v];
                const int side = t1 > t0 ? 1 : 0;
                for (int v : comp) pick[v] = color[v] == side;
            } else {
                std::vector<int> ord(comp);
                std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return touches[x] > touches[y]; });
                for (int v : ord) {
                    bool ok = true;
                    for (int u : adj[v]) ok &= !pick[u];
                    pick[v] = ok;
                }
            }
        }
        for (int v = 0; v < nq; ++v)
            if (pick[v] && touches[v] >= 2) resident.push_back(v);
        std::stable_sort(resident.begin(), resident.end(), [&](int x, int y) { return touches[x] > touches[y]; });
        if (resident.size() > 256) resident.resize(256);
        if (resident.empty()) res_form = false;
    }
    std::vector<int> res_ord(nq, -1);
    int RC = 0;
    // per layer, per resident ordinal: (code, partner local column)
    std::vector<std::vector<std::pair<uint8_t, int>>> rops;
    if (res_form) {
        // Owners: ordinals sorted by their gate signature, so lanes of one
        // slot tend to run the same code (no divergence).
        std::vector<std::string> sig(nq);
        for (int l = 0; l < nl; ++l)
            for (const SegGate &g : L[l].gates) {
                const int32_t code = g.code_rec & 15;
                sig[g.a] += (char)('a' + code * 2);
                if (code == OP_CX || code == OP_CZ) sig[g.b] += (char)('a' + code * 2 + 1);
            }
        std::stable_sort(resident.begin(), resident.end(), [&](int x, int y) { return sig[x] < sig[y]; });
        for (size_t i = 0; i < resident.size(); ++i) res_ord[resident[i]] = (int)i;
        const int need = (int)((resident.size() + 31) / 32);
        RC = need <= 2 ? 2 : need <= 4 ? 4 : 8;
        rops.assign(nl, std::vector<std::pair<uint8_t, int>>(resident.size(), {RS_NOP, 0}));
        for (int l = 0; l < nl; ++l) {
            std::vector<SegGate> free_gates;
            for (const SegGate &g : L[l].gates) {
                const int32_t code = g.code_rec & 15;
                const int ra = res_ord[g.a];
                const int rb = (code == OP_CX || code == OP_CZ) ? res_ord[g.b] : -1;
                if (ra >= 0 && (code == OP_H || code == OP_S)) {
                    rops[l][ra] = {code == OP_H ? RS_H : RS_S, 0};
                } else if (ra >= 0 && (code == OP_CX || code == OP_CZ)) {
                    rops[l][ra] = {code == OP_CX ? RS_CX_CTRL : RS_CZ, g.b};
                } else if (rb >= 0) {
                    rops[l][rb] = {code == OP_CX ? RS_CX_TGT : RS_CZ, g.a};
                } else {
                    free_gates.push_back(g);
                }
            }
            L[l].gates = free_gates;
        }
    }

    // ---- propagated Paulis of channel components and sign ops (local
    // columns; mapped to tile positions after the permutation below)
    std::vector<std::vector<std::pair<int, uint8_t>>> props;  // bits: 1 = x, 2 = z
    if (res_form) {
        std::vector<std::vector<int>> gate_at(nl, std::vector<int>(nq, -1));
        for (int l = 0; l < nl; ++l)
            for (size_t gi = 0; gi < all_gates[l].size(); ++gi) {
                const SegGate &g = all_gates[l][gi];
                gate_at[l][g.a] = (int)gi;
                const int32_t code = g.code_rec & 15;
                if (code == OP_CX || code == OP_CZ) gate_at[l][g.b] = (int)gi;
            }
        auto propagate = [&](int col, uint8_t bits, int from) {
            std::map<int, uint8_t> p;
            if (col >= 0 && bits) p[col] = bits;
            for (int l = from + 1; l < nl && !p.empty(); ++l) {
                std::set<int> gs;
                for (auto &kv : p)
                    if (gate_at[l][kv.first] >= 0) gs.insert(gate_at[l][kv.first]);
                for (int gi : gs) {
                    const SegGate &g = all_gates[l][gi];
                    const int32_t code = g.code_rec & 15;
                    auto get = [&](int q) { auto it = p.find(q); return it == p.end() ? (uint8_t)0 : it->second; };
                    const uint8_t va = get(g.a);
                    const int xa = va & 1, za = (va >> 1) & 1;
                    if (code == OP_H) {
                        p[g.a] = (uint8_t)(za | (xa << 1));
                    } else if (code == OP_S) {
                        p[g.a] = (uint8_t)(xa | ((za ^ xa) << 1));
                    } else {
                        const uint8_t vb = get(g.b);
                        const int xb = vb & 1, zb = (vb >> 1) & 1;
                        if (code == OP_CX) {  // X_c -> X_c X_t, Z_t -> Z_c Z_t
                            p[g.a] = (uint8_t)(xa | ((za ^ zb) << 1));
                            p[g.b] = (uint8_t)((xb ^ xa) | (zb << 1));
                        } else {  // CZ: X_a -> X_a Z_b
                            p[g.a] = (uint8_t)(xa | ((za ^ xb) << 1));
                            p[g.b] = (uint8_t)(xb | ((zb ^ xa) << 1));
                        }
                    }
                }
                for (auto it = p.begin(); it != p.end();) it = it->second ? std::next(it) : p.erase(it);
            }
            return std::vector<std::pair<int, uint8_t>>(p.begin(), p.end());
        };
        for (int l = 0; l < nl; ++l)
            for (const NoiseSlot &sl : L[l].slots) {
                props.push_back(propagate(sl.a, 1, l));
                props.push_back(propagate(sl.a, 2, l));
                props.push_back(propagate(sl.b, 1, l));
                props.push_back(propagate(sl.b, 2, l));
            }
        for (int l = 0; l < nl; ++l)
            for (const SegSign &sg : L[l].signs)
                props.push_back(propagate(sg.a, sg.kind == SIGN_Z ? 2 : sg.kind == SIGN_Y ? 3 : 1, l));
        for (auto &pr : props)
            if (pr.size() > 255) res_form = false;
    }

    // Tile positions: a permutation of the columns.  Default form: a local
    // search that swaps the positions of two columns whenever that keeps or
    // lowers (lane groups needed summed over the gate runs, squared residue
    // counts summed), until the groups reach their lower bound, the sum of
    // ceil(gates / 8) over the runs.  Resident form: identity or one of a few
    // seeded shuffles, whichever needs the fewest groups plus bank conflicts
    // of the owners' partner cells.
    auto remap = [](const std::vector<SegGate> &gs, const std::vector<int> &perm) {
        std::vector<SegGate> out(gs);
        for (SegGate &g : out) {
            g.a = (uint16_t)perm[g.a];
            g.b = (uint16_t)perm[g.b];
        }
        return out;
    };
    auto splitmix = [](uint64_t &st) {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    std::vector<int> best(nq);
    for (int i = 0; i < nq; ++i) best[i] = i;
    if (res_form) {
        auto groups_needed = [&](const std::vector<int> &perm) {
            size_t total = 0;
            for (int l = 0; l < nl; ++l)  // per (layer, slot, quarter-warp): largest residue multiplicity
                for (size_t base = 0; base < resident.size(); base += 8) {
                    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0}, mx = 0;
                    for (size_t o = base; o < std::min(resident.size(), base + 8); ++o)
                        if (rops[l][o].first >= RS_CX_CTRL) mx = std::max(mx, ++cnt[perm[rops[l][o].second] & 7]);
                    total += (size_t)mx;
                }
            for (size_t l = 0; l < L.size(); ++l)
                for (int32_t code : {(int32_t)OP_H, (int32_t)OP_S, (int32_t)OP_CX, (int32_t)OP_CZ}) {
                    std::vector<SegGate> gs;
                    for (const SegGate &g : L[l].gates)
                        if ((g.code_rec & 15) == code) gs.push_back(g);
                    if (!gs.empty()) total += (size_t)lane_groups_needed(remap(gs, perm), code == OP_CX || code == OP_CZ);
                }
            return total;
        };
        size_t best_cost = groups_needed(best);
        for (uint64_t seed = 1; seed <= 12 && nq > 8; ++seed) {
            std::vector<int> perm(nq);
            for (int i = 0; i < nq; ++i) perm[i] = i;
            uint64_t st = seed * 0x9E3779B97F4A7C15ull;
            for (int i = nq - 1; i > 0; --i) std::swap(perm[i], perm[(int)(splitmix(st) % (uint64_t)(i + 1))]);
            const size_t cost = groups_needed(perm);
            if (cost < best_cost) {
                best_cost = cost;
                best = perm;
            }
        }
    } else if (nq > 8) {
        struct RunCount {
            int cnt[2][8];
        };
        std::vector<RunCount> rc;
        std::vector<std::vector<std::pair<int, int>>> app(nq);  // column -> (run, side)
        long lower = 0;
        for (size_t l = 0; l < L.size(); ++l)
            for (int32_t code : {(int32_t)OP_H, (int32_t)OP_S, (int32_t)OP_CX, (int32_t)OP_CZ}) {
                const bool two = code == OP_CX || code == OP_CZ;
                const int ri = (int)rc.size();
                int ng = 0;
                for (const SegGate &g : L[l].gates)
                    if ((g.code_rec & 15) == code) {
                        app[g.a].emplace_back(ri, 0);
                        if (two) app[g.b].emplace_back(ri, 1);
                        ++ng;
                    }
                if (ng == 0) continue;
                rc.push_back(RunCount{});
                lower += (ng + 7) / 8;
            }
        for (int col = 0; col < nq; ++col)
            for (auto &e : app[col]) rc[(size_t)e.first].cnt[e.second][best[col] & 7]++;
        auto groups = [&](int ri) {
            int D = 0;
            for (int sd = 0; sd < 2; ++sd)
                for (int r = 0; r < 8; ++r) D = std::max(D, rc[(size_t)ri].cnt[sd][r]);
            return D;
        };
        auto squares = [&](int ri) {
            long q = 0;
            for (int sd = 0; sd < 2; ++sd)
                for (int r = 0; r < 8; ++r) q += (long)rc[(size_t)ri].cnt[sd][r] * rc[(size_t)ri].cnt[sd][r];
            return q;
        };
        long cost = 0;
        for (int ri = 0; ri < (int)rc.size(); ++ri) cost += groups(ri);
        std::vector<int> stamp(rc.size(), -1), touched;
        uint64_t st = 0x5EEDull;
        const long iters = std::min<long>(400000, 100L * nq);
        for (long it = 0; it < iters && cost > lower; ++it) {
            const int x = (int)(splitmix(st) % (uint64_t)nq), y = (int)(splitmix(st) % (uint64_t)nq);
            const int rx = best[x] & 7, ry = best[y] & 7;
            if (rx == ry) continue;
            touched.clear();
            for (int v : {x, y})
                for (auto &e : app[v])
                    if (stamp[(size_t)e.first] != (int)it) {
                        stamp[(size_t)e.first] = (int)it;
                        touched.push_back(e.first);
                    }
            long g0 = 0, q0 = 0, g1 = 0, q1 = 0;
            for (int ri : touched) {
                g0 += groups(ri);
                q0 += squares(ri);
            }
            auto move = [&](int v, int from, int to) {
                for (auto &e : app[v]) {
                    rc[(size_t)e.first].cnt[e.second][from]--;
                    rc[(size_t)e.first].cnt[e.second][to]++;
                }
            };
            move(x, rx, ry);
            move(y, ry, rx);
            for (int ri : touched) {
                g1 += groups(ri);
                q1 += squares(ri);
            }
            if (g1 < g0 || (g1 == g0 && q1 <= q0)) {
                std::swap(best[x], best[y]);
                cost += g1 - g0;
            } else {
                move(x, ry, rx);
                move(y, rx, ry);
            }
        }
    }
    {
        std::vector<int32_t> cols(nq);
        for (int i = 0; i < nq; ++i) cols[best[i]] = seg.cols[i];
        seg.cols = cols;
    }
    for (size_t l = 0; l < L.size(); ++l) {
        L[l].gates = remap(L[l].gates, best);
        for (SegSign &sg : L[l].signs) sg.a = (uint16_t)best[sg.a];
        for (NoiseSlot &sl : L[l].slots) {
            sl.a = best[sl.a];
            if (sl.b >= 0) sl.b = best[sl.b];
        }
    }
    for (size_t l = 0; l < L.size(); ++l) {
        SegLayer ly{};
        ly.r0 = (int32_t)seg.runs.size();
        for (int32_t code : {(int32_t)OP_H, (int32_t)OP_S, (int32_t)OP_CX, (int32_t)OP_CZ, (int32_t)-1}) {
            std::vector<SegGate> gs;
            for (const SegGate &g : L[l].gates) {
                const int32_t gc = g.code_rec & 15;
                const bool uniform = gc == OP_H || gc == OP_S || gc == OP_CX || gc == OP_CZ;
                if ((code >= 0 && gc == code) || (code < 0 && !uniform)) gs.push_back(g);
            }
            if (gs.empty()) continue;
            SegRun run{code, (int32_t)seg.gates.size(), 0, 0};
            if (code < 0) {
                seg.gates.insert(seg.gates.end(), gs.begin(), gs.end());
            } else {
                for (auto &grp : lane_groups(gs, code == OP_CX || code == OP_CZ, nq, code))
                    seg.gates.insert(seg.gates.end(), grp.begin(), grp.end());
            }
            run.g1 = (int32_t)seg.gates.size();
            seg.runs.push_back(run);
        }
        ly.r1 = (int32_t)seg.runs.size();
        ly.s0 = (int32_t)seg.signs.size();
        if (res_form) {  // after the last layer, in this order (propagated Pauli 4*nslots + k)
            seg.signs.insert(seg.signs.end(), L[l].signs.begin(), L[l].signs.end());
        } else {
            // interleave residues so 8 consecutive sign ops read distinct bank groups
            std::vector<SegSign> byres[8];
            for (const SegSign &sg : L[l].signs) byres[sg.a & 7].push_back(sg);
            for (bool more = true; more;) {
                more = false;
                for (int r8 = 0; r8 < 8; ++r8)
                    if (!byres[r8].empty()) {
                        seg.signs.push_back(byres[r8].back());
                        byres[r8].pop_back();
                        more = true;
                    }
            }
        }
        ly.s1 = (int32_t)seg.signs.size();
        seg.layers.push_back(ly);
        seg.slots.insert(seg.slots.end(), L[l].slots.begin(), L[l].slots.end());
        seg.slot_op.insert(seg.slot_op.end(), L[l].slot_ops.begin(), L[l].slot_ops.end());
    }
    {  // record slots renumbered in sign order: the lanes of a sign batch read consecutive record words
        std::vector<int32_t> order;
        order.reserve(seg.recsig_rec.size());
        for (SegSign &sg : seg.signs)
            if (sg.kind == SIGN_REC_X) {
                order.push_back(seg.recsig_rec[(size_t)sg.rec]);
                sg.rec = (int32_t)order.size() - 1;
            }
        seg.recsig_rec = std::move(order);
    }
    if (res_form) {
        seg.res_slots = RC;
        seg.res_cols.assign((size_t)RC * 32, (uint16_t)0xFFFF);
        for (size_t o = 0; o < resident.size(); ++o) seg.res_cols[o] = (uint16_t)best[resident[o]];
        seg.res_ops.assign((size_t)nl * RC * 32, ResOp{0, RS_NOP, 0});
        for (int l = 0; l < nl; ++l)
            for (size_t o = 0; o < resident.size(); ++o) {
                const auto &op = rops[l][o];
                if (op.first == RS_NOP) continue;
                seg.res_ops[(size_t)l * RC * 32 + o] =
                    ResOp{(uint16_t)(op.first >= RS_CX_CTRL ? best[op.second] : 0), op.first, 0};
            }
        for (const auto &pr : props) {
            seg.prop_desc.push_back(((uint32_t)seg.prop_sup.size() << 8) | (uint32_t)pr.size());
            for (const auto &e : pr)
                seg.prop_sup.push_back((uint32_t)best[e.first] | ((e.second & 1) ? PROP_X : 0u) |
                                       ((e.second & 2) ? PROP_Z : 0u));
        }
        if (seg.prop_sup.empty()) seg.prop_sup.push_back(0);
    }
    (void)rec_of;
    return OK;
}

// Largest shared-memory footprint of any segment launch for a tile shape.
size_t max_seg_smem(const ps_circuit *c, int rows, int bw) {
    size_t m = 0;
    for (const SegHost &sg : c->segs)
        m = std::max(m, segment_launch_smem((int)sg.layers.size(), (int)sg.runs.size(), (int)sg.gates.size(),
                                            (int)sg.signs.size(), (int)sg.cols.size(), (int)sg.recsig_rec.size(),
                                            rows, bw, sg.res_slots));
    return m;
}

void pick_tile(ps_circuit *c) {
    ps_circuit_options &o = c->opts;
    const ps_state *h = c->h;
    if (o.seg_rows <= 0) o.seg_rows = 1;
    if (o.seg_words <= 0) {
        int bw = 8;
        while (bw > 1 && (max_seg_smem(c, o.seg_rows, bw) > 200 * 1024 || bw > h->w)) bw >>= 1;
        o.seg_words = bw;
    }
    if (o.seg_threads <= 0) o.seg_threads = std::min(256, std::max(32, 32 * o.seg_rows * o.seg_words));
}

// Optional per-launch timing: an event pair around every launch, by kind.
struct Profiler {
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    cudaStream_t st;
    int begin(int kind) {
        cudaEvent_t a, b;
        PS_CUDA(cudaEventCreate(&a));
        PS_CUDA(cudaEventCreate(&b));
        PS_CUDA(cudaEventRecord(a, st));
        marks.push_back({kind, {a, b}});
        return OK;
    }
    int end() {
        PS_CUDA(cudaEventRecord(marks.back().second.second, st));
        return OK;
    }
    ~Profiler() {
        for (auto &m : marks) {
            cudaEventDestroy(m.second.first);
            cudaEventDestroy(m.second.second);
        }
    }
};

enum ProfKind { P_INIT = 0, P_SAMPLE = 1, P_SEGMENT = 2, P_MEASURE = 3, P_GATE = 4, P_CHANNEL = 5, P_FRAME = 6, P_BROADCAST = 7 };

// Enqueues plan steps [from, to) on `st`.
// The per-shot plan's device schedules and channel scratch: built on first
// use -- a run without reset, measurement statistics, the tile tuner, or at
// compile time when the shared-x/z plan does not apply -- so circuits that
// only run from |0...0> in the shared-x/z plan never upload them.  Not
// during stream capture (it uploads with synchronous copies).
int build_segments_dev(ps_circuit *c);
int ensure_segments_dev(ps_circuit *c) {
    if (c->seg_dev_ready || c->opts.mode != PS_MODE_FUSED) return OK;
    if (c->h->signs_only) return fail(E_STATE, "a signs-only state runs only the shared-x/z plan");
    if (c->seg_dev_status >= 0)
        return fail(c->seg_dev_status, "the per-shot plan of this circuit does not fit its kernels");
    c->seg_dev_status = build_segments_dev(c);
    c->seg_dev_ready = c->seg_dev_status == OK;
    return c->seg_dev_status;
}

int build_segments_dev(ps_circuit *c) {
    ps_state *h = c->h;
    c->entry_cap = (int32_t)std::max<size_t>(1, c->max_slots);
    void *p = nullptr;
    if (dev_alloc(h, &p, (size_t)c->entry_cap * h->w * sizeof(NoiseEntry)) != OK)
        return fail(E_NOMEM, "device allocation of channel entries failed");
    c->owned.push_back(p);
    c->d_entries = (NoiseEntry *)p;
    if (dev_alloc(h, &p, (size_t)h->w * sizeof(int32_t)) != OK) return E_NOMEM;
    c->owned.push_back(p);
    c->d_entry_count = (int32_t *)p;
    if (dev_alloc(h, &p, (size_t)c->entry_cap * h->w * 4 * sizeof(u64)) != OK)
        return fail(E_NOMEM, "device allocation of channel sampling scratch failed");
    c->owned.push_back(p);
    c->d_dense = (u64 *)p;
    for (SegHost &sg : c->segs) {
        SegmentDev d{};
        SegLayer *dl;
        SegRun *drn;
        SegGate *dg;
        SegSign *ds;
        int32_t *dc;
        NoiseSlot *dsl;
        int32_t *drr;
        if (upload(h, c->owned, sg.layers, &dl) || upload(h, c->owned, sg.runs, &drn) || upload(h, c->owned, sg.gates, &dg) ||
            upload(h, c->owned, sg.signs, &ds) ||
            upload(h, c->owned, sg.cols, &dc) || upload(h, c->owned, sg.slots, &dsl) ||
            upload(h, c->owned, sg.recsig_rec, &drr))
            return E_CUDA;
        d.recsig_rec = drr;
        d.nrecsig = (int32_t)sg.recsig_rec.size();
        d.word_vector = c->opts.seg_resident == 2 ? 1 : 0;
        if (sg.res_slots > 0) {
            uint16_t *drc;
            ResOp *dro;
            uint32_t *dpd, *dps;
            if (upload(h, c->owned, sg.res_cols, &drc) || upload(h, c->owned, sg.res_ops, &dro) ||
                upload(h, c->owned, sg.prop_desc, &dpd) || upload(h, c->owned, sg.prop_sup, &dps))
                return E_CUDA;
            d.res_slots = sg.res_slots;
            d.res_cols = drc;
            d.res_ops = dro;
            d.prop_desc = dpd;
            d.prop_sup = dps;
        }
        d.layers = dl;
        d.nlayers = (int32_t)sg.layers.size();
        d.runs = drn;
        d.nruns = (int32_t)sg.runs.size();
        d.gates = dg;
        d.signs = ds;
        d.cols = dc;
        d.nq = (int32_t)sg.cols.size();
        d.ngates = (int32_t)sg.gates.size();
        d.nsigns = (int32_t)sg.signs.size();
        d.slots = dsl;
        d.nslots = (int32_t)sg.slots.size();
        d.thr = c->d_thr;
        d.entries = sg.slots.empty() ? nullptr : c->d_entries;
        d.entry_count = c->d_entry_count;
        d.cap = c->entry_cap;
        d.dense = c->d_dense;
        sg.dev = d;
        if (segment_launch_smem(d.nlayers, d.nruns, d.ngates, d.nsigns, d.nq, d.nrecsig, c->opts.seg_rows,
                                c->opts.seg_words, d.res_slots) > kSegSmemMax)
            return fail(E_ARG, "segment schedule and tile do not fit in shared memory");
    }
    return OK;
}

int enqueue_steps(ps_circuit *c, cudaStream_t st, size_t from, size_t to, Profiler *prof = nullptr) {
    ps_state *h = c->h;
    auto timed = [&](int kind, auto &&launch) -> int {
        if (prof && prof->begin(kind) != OK) return E_CUDA;
        int rc = launch();
        if (prof && rc == OK && prof->end() != OK) return E_CUDA;
        return rc;
    };
    for (size_t i = from; i < to && i < c->steps.size(); ++i) {
        const Step &s = c->steps[i];
        int rc = OK;
        switch (s.kind) {
        case K_GATE:
            rc = timed(P_GATE, [&] {
                return launch_gate_on(st, h, s.code, s.a, s.b,
                                      s.rec >= 0 ? h->recs[(size_t)c->rec_ids[(size_t)s.rec]].res : nullptr);
            });
            break;
        case K_CHANNEL:
            rc = timed(P_CHANNEL, [&] {
                return launch_channel_apply(st, h, s.a, s.b, c->d_thr + s.first, s.count, c->d_psurv + 64 * s.table,
                                            c->pest[(size_t)s.table], s.event, c->d_params);
            });
            break;
        case K_MEAS:
            rc = timed(P_MEASURE, [&] {
                return launch_measure_list(st, h->X, h->Z, h->R, h->n, h->w, c->d_meas + s.first, s.count,
                                           (uint64_t)h->seed, (uint64_t)h->word_base, c->d_params,
                                           c->opts.meas_words);
            });
            break;
        case K_SEGMENT: {
            const SegHost &sg = c->segs[(size_t)s.first];
            if (!sg.slots.empty()) rc = timed(P_SAMPLE, [&] { return launch_noise_sample(st, sg.dev, h->w, c->d_params); });
            if (rc == OK)
                rc = timed(P_SEGMENT, [&] {
                    return launch_segment(st, h->X, h->Z, h->R, h->n, h->w, sg.dev, c->opts.seg_rows,
                                          c->opts.seg_words, c->opts.seg_threads, c->d_recs);
                });
            break;
        }
        default: break;
        }
        if (rc != OK) return rc;
    }
    return OK;
}

// The device job of a compiled circuit's sign program (all but the tables
// the caller uploads: ranges, channel records, channel tables, survival
// products): one range per launch range of the program, and the
// shared-memory layout.  A range's ops and measurement tab words are staged
// in shared memory while the staging buffers stay within kFrameStageMax and
// the sign kernel's shared memory; ranges that would need more read them
// from global memory.  E_ARG: the program does not fit this kernel (the
// per-shot plan runs instead).
int frame_job_ranges(ps_circuit *c, FrameJobDev &job, std::vector<FrameRangeDev> &ranges,
                     std::vector<FrameSlotDev> &slots, std::vector<uint32_t> &s64, std::vector<uint32_t> &events,
                     std::vector<int32_t> &nv_range, std::vector<FrameChanTab> &ctabs,
                     std::vector<uint32_t> &surv) {
    ps_state *h = c->h;
    const FrameProgram &P = c->fprog;
    ranges.clear();
    uint32_t max_rand = 0, max_scratch = 0, max_slots = 0;
    // channel records (indexed like slot_off) and the distinct tables
    slots.clear();
    nv_range.clear();
    events.assign(P.slot_off.size(), 0u);
    s64.clear();
    std::map<int32_t, uint32_t> table_of;
    ctabs.clear();
    surv.clear();
    for (const FrameProgram::Launch &L : P.launches) {
        max_rand = std::max(max_rand, L.nrand);
        max_scratch = std::max(max_scratch, L.scratch);
        FrameRangeDev r{};
        r.op0 = L.op0;
        r.op1 = L.op1;
        r.rand0 = L.rand0;
        r.nrand = L.nrand;
        if (L.seg >= 0) {
            if (L.op0 >= L.op1 || (P.ops[L.op0].kind & 0xFFu) != F_NOISE)
                return fail(E_ARG, "shared-x/z plan: a sampled range must start with its noise");
            const SegHost &sg = c->segs[(size_t)L.seg];
            r.nslots = (int32_t)sg.slots.size();
            r.slot_base = (uint32_t)P.ops[L.op0].arg;
            max_slots = std::max(max_slots, (uint32_t)r.nslots);
            if ((size_t)r.slot_base + (size_t)r.nslots >= events.size())
                return fail(E_ARG, "shared-x/z plan: channel table out of range");
            // this segment's channel records from a 16-byte boundary, padded to one
            r.rec_base = (uint32_t)slots.size();
            slots.resize(slots.size() + (((size_t)r.nslots + 1) & ~(size_t)1), FrameSlotDev{0u, kFrameNoHit});
            // this segment's S_64 words from a 16-byte boundary, padded to one
            r.s64_base = (uint32_t)s64.size();
            s64.resize(s64.size() + (((size_t)r.nslots + 3) & ~(size_t)3), 0xFFFFFFFFu);
            for (int32_t q = 0; q < r.nslots; ++q) {
                const NoiseSlot &sl = sg.slots[(size_t)q];
                auto it = table_of.find(sl.thr_off);
                if (it == table_of.end()) {
                    if (ctabs.size() >= kFrameMaxTables) return fail(E_ARG, "shared-x/z plan: too many channel tables");
                    it = table_of.emplace(sl.thr_off, (uint32_t)ctabs.size()).first;
                    FrameChanTab ct{};
                    ct.thr_off = sl.thr_off;
                    ct.count = sl.count;
                    ct.surv_off = (uint32_t)surv.size();
                    ct.est = channel_est_factors(c->thr_host[(size_t)(sl.thr_off + sl.count - 1)], sl.count);
                    ctabs.push_back(ct);
                    surv.resize(surv.size() + 64);
                    channel_surv_table(c->thr_host[(size_t)(sl.thr_off + sl.count - 1)], &surv[surv.size() - 64]);
                }
                const uint32_t t0 = P.slot_off[(size_t)r.slot_base + (size_t)q];
                const uint32_t len = P.slot_off[(size_t)r.slot_base + (size_t)q + 1] - t0;
                if (len > kFrameMaxSlotRows) return fail(E_ARG, "shared-x/z plan: a channel flips too many rows");
                const bool never = c->thr_host[(size_t)(sl.thr_off + sl.count - 1)] == 0;
                FrameSlotDev &d = slots[(size_t)r.rec_base + (size_t)q];
                d.t0 = t0;
                d.lt = len << 12 | (never ? kFrameNoHit : it->second);
                events[(size_t)r.slot_base + (size_t)q] = sl.event;
                s64[(size_t)r.s64_base + (size_t)q] =
                    never ? 0xFFFFFFFFu : (uint32_t)c->thr_host[(size_t)(sl.thr_off + sl.count)];
            }
        }
        r.ev0 = -1;
        r.nv = -1;
        if (r.nslots > 0) {  // consecutive events: the kernel draws first draws four channels a block
            bool run = true;
            for (int32_t q = 1; q < r.nslots && run; ++q)
                run = events[(size_t)r.slot_base + q] == events[(size_t)r.slot_base] + (uint32_t)q;
            if (run && events[(size_t)r.slot_base] <= 0x7FFFFFFFu) r.ev0 = (int32_t)events[(size_t)r.slot_base];
        }
        if (r.nslots > 0) {  // its noise vectors: block nv of nvec
            r.nv = (int32_t)nv_range.size();
            nv_range.push_back((int32_t)ranges.size());
        }
        r.tab0a = L.tab0 & ~3u;
        r.ntab16 = (((L.tab1 + 3u) & ~3u) - r.tab0a) / 4;
        ranges.push_back(r);
    }
    if (ranges.empty()) return fail(E_ARG, "shared-x/z plan: empty program");
    if (slots.empty()) slots.resize(2, FrameSlotDev{0u, kFrameNoHit});
    if (s64.empty()) s64.resize(4, 0xFFFFFFFFu);
    job.R = h->R;
    job.n = h->n;
    job.w = h->w;
    job.ops = c->d_fops;
    job.tab = c->d_ftab;
    job.nranges = (int32_t)ranges.size();
    job.rand_meas = c->d_frand;
    job.meas = c->d_meas;
    job.rec = c->d_res_block;
    job.nm = (int64_t)c->meas.size();
    job.thr = c->d_thr;
    job.rp = c->d_params;
    job.max_rand = max_rand;
    job.max_scratch = max_scratch;
    job.max_slots = max_slots;
    job.n_ctab = (uint32_t)ctabs.size();
    job.n_thr = (uint32_t)c->thr_host.size();
    job.n_surv = (uint32_t)surv.size();
    job.nnv = (int32_t)nv_range.size();
    job.stage_tabs = (size_t)job.n_ctab * sizeof(FrameChanTab) + (size_t)job.n_thr * 8 + (size_t)job.n_surv * 4 <= kFrameTabStage ? 1u : 0u;
    // staging: drop the largest staged range until the buffers fit, each
    // within kFrameStageMax and both within what the rest of the sign
    // kernel's shared memory leaves
    job.stage_u32 = 0;
    job.max_ops = 0;
    const size_t rest = frame_job_smem(job) + 64;  // + alignment of the two buffers
    const size_t stage_max = rest < kSegSmemMax ? std::min(kFrameStageMax, (kSegSmemMax - rest) / 2 & ~(size_t)15) : 0;
    std::vector<char> on(ranges.size(), 1);
    for (;;) {
        uint32_t tab = 0, nops = 0;
        size_t worst = ranges.size(), worst_need = 0;
        for (size_t i = 0; i < ranges.size(); ++i) {
            if (!on[i]) continue;
            tab = std::max(tab, 4 * ranges[i].ntab16);
            nops = std::max(nops, ranges[i].op1 - ranges[i].op0);
            const size_t need = (size_t)ranges[i].ntab16 * 16 + (size_t)(ranges[i].op1 - ranges[i].op0) * sizeof(FrameOp);
            if (need >= worst_need) {
                worst = i;
                worst_need = need;
            }
        }
        job.stage_u32 = tab;
        job.max_ops = nops;
        if (worst == ranges.size() || (size_t)tab * 4 + (size_t)nops * sizeof(FrameOp) <= stage_max) break;
        on[worst] = 0;
    }
    for (size_t i = 0; i < ranges.size(); ++i) ranges[i].stage = on[i] ? 1u : 0u;
    if (frame_job_smem(job) > kSegSmemMax) return fail(E_ARG, "sign program does not fit in shared memory");
    if (job.nnv > 0 && noise_job_smem(job) > kSegSmemMax) return fail(E_ARG, "channel noise does not fit in shared memory");
    return OK;
}

// The shared-x/z plan of a run from |0...0>: the noise vectors of every range
// and shot-word, then the whole sign program as one launch, with the
// broadcast of the final x / z bits (host-known, so it needs nothing else)
// beside them on a side stream, joined back at the end.  Profiled, the three
// run one after the other.
struct EventPair {
    cudaEvent_t a = nullptr, b = nullptr;
    EventPair() {
        if (cudaEventCreate(&a) != cudaSuccess) a = nullptr;
        if (cudaEventCreate(&b) != cudaSuccess) b = nullptr;
    }
    ~EventPair() {
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
    bool ok() const { return a && b; }
};

int enqueue_frame_table(const FrameTable &t, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                        int warps, int bctas, Profiler *prof) {
    auto timed = [&](int kind, auto &&launch) -> int {
        if (prof && prof->begin(kind) != OK) return E_CUDA;
        int rc = launch();
        if (prof && rc == OK && prof->end() != OK) return E_CUDA;
        return rc;
    };
    NvtxRange range("ps shared-x/z run (" + std::to_string(t.njobs) + " jobs)");
    if (prof || !side || t.chunks == 0) {
        int rc = timed(P_SAMPLE, [&] {
            NvtxRange r("ps noise vectors");
            return launch_noise_vectors(st, t);
        });
        if (rc == OK) rc = timed(P_FRAME, [&] {
            NvtxRange r("ps sign program");
            return launch_frame_run(st, t, warps);
        });
        if (rc != OK) return rc;
        return timed(P_BROADCAST, [&] {
            NvtxRange r("ps x/z broadcast");
            return launch_broadcast_jobs(st, t, bctas);
        });
    }
    // The broadcast runs beside the noise vectors and the sign program, at
    // the highest priority, so that its CTAs hold their SMs from the start.
    PS_CUDA(cudaEventRecord(fork, st));
    PS_CUDA(cudaStreamWaitEvent(side, fork, 0));
    int rc;
    {
        NvtxRange r("ps x/z broadcast");
        rc = launch_broadcast_jobs(side, t, bctas);
    }
    if (rc == OK) {
        NvtxRange r("ps noise vectors");
        rc = launch_noise_vectors(st, t);
    }
    if (rc != OK) return rc;
    {
        NvtxRange r("ps sign program");
        rc = launch_frame_run(st, t, warps);
    }
    if (rc != OK) return rc;
    PS_CUDA(cudaEventRecord(join, side));
    PS_CUDA(cudaStreamWaitEvent(st, join, 0));
    return OK;
}

int enqueue_frame(ps_circuit *c, cudaStream_t st, Profiler *prof) {
    return enqueue_frame_table(c->ftable, st, c->fstream, c->fev[0], c->fev[1], c->opts.frame_warps,
                               c->opts.bcast_ctas, prof);
}

// The fastest (sign-kernel warps, broadcast CTAs per SM) for a table: each
// candidate runs twice (the first warms up), timed with events on st.  The
// run parameters must be on the device already; the signs, records, noise
// vectors and x / z the runs write are left behind.
int tune_frame_table(const FrameTable &t, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                     int *warps, int *bctas, double *best_ms) {
    EventPair ev;
    if (!ev.ok()) return cuda_fail(cudaGetLastError(), "cudaEventCreate");
    float best = 3.0e38f;
    const int wc[] = {8, 4};
    const int bc[] = {1, 2};
    for (int fw : wc)
        for (int b : bc) {
            if (t.chunks == 0 && b != 1) continue;  // no broadcast
            float ms = 0.f;
            for (int rep = 0; rep < 2; ++rep) {
                PS_CUDA(cudaEventRecord(ev.a, st));
                int rc = enqueue_frame_table(t, st, side, fork, join, fw, b, nullptr);
                if (rc != OK) return rc;
                PS_CUDA(cudaEventRecord(ev.b, st));
                PS_CUDA(cudaEventSynchronize(ev.b));
                PS_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
            }
            if (ms < best) {
                best = ms;
                *warps = fw;
                *bctas = b;
            }
        }
    if (best_ms) *best_ms = best;
    return OK;
}

int enqueue_plan(ps_circuit *c, cudaStream_t st, bool reset, Profiler *prof = nullptr) {
    if (reset && c->frame_ok && !c->force_per_shot) return enqueue_frame(c, st, prof);
    {
        int rc = ensure_segments_dev(c);  // (captures call it before they begin)
        if (rc != OK) return rc;
    }
    if (reset) {
        if (prof && prof->begin(P_INIT) != OK) return E_CUDA;
        int rc = launch_init_zero_on(st, c->h);
        if (rc != OK) return rc;
        if (prof && prof->end() != OK) return E_CUDA;
    }
    return enqueue_steps(c, st, 0, c->steps.size(), prof);
}

// Captures the plan of runs without (reset = 0) or with the reset into its
// CUDA graph, replacing an earlier one.
int capture_graph(ps_circuit *c, int reset) {
    if (c->exec[reset]) cudaGraphExecDestroy(c->exec[reset]);
    if (c->graph[reset]) cudaGraphDestroy(c->graph[reset]);
    c->exec[reset] = nullptr;
    c->graph[reset] = nullptr;
    cudaStream_t cs;
    PS_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = e == cudaSuccess ? enqueue_plan(c, cs, reset != 0) : cuda_fail(e, "cudaStreamBeginCapture");
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc != OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
    c->graph[reset] = g;
    // node priorities kept: the broadcast's CTAs go first
    e = cudaGraphInstantiateWithFlags(&c->exec[reset], g, cudaGraphInstantiateFlagUseNodePriority);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    return OK;
}

// Captures both graphs.  Without reset, a circuit with the shared-x/z plan
// runs its per-shot plan, which is built and captured at the first such run
// (unless it is built already).  A register the per-shot kernels cannot take
// (more qubits than the measurement kernel holds) still runs from |0...0> in
// the shared-x/z plan; a run without reset reports the error.
int capture_graphs(ps_circuit *c) {
    for (int reset = 0; reset < 2; ++reset) {
        if (c->exec[reset]) cudaGraphExecDestroy(c->exec[reset]);
        if (c->graph[reset]) cudaGraphDestroy(c->graph[reset]);
        c->exec[reset] = nullptr;
        c->graph[reset] = nullptr;
        if (reset == 0 && c->h->signs_only) continue;  // runs only from |0...0>
        if (reset == 0 && c->frame_ok && !c->seg_dev_ready) continue;
        if (reset == 0 || !c->frame_ok) {
            int rc = ensure_segments_dev(c);  // (uploads: not inside the capture)
            if (rc != OK) {
                if (reset == 0 && c->frame_ok && rc == E_ARG) continue;
                return rc;
            }
        }
        int rc = capture_graph(c, reset);
        if (rc != OK) {
            if (reset == 0 && c->frame_ok && rc == E_ARG) continue;
            return rc;
        }
    }
    return OK;
}

// Host bookkeeping of one run: records go stale, the event counter advances;
// returns the run's parameters.
RunParams begin_run(ps_circuit *c, bool reset) {
    ps_state *h = c->h;
    for (int64_t id : c->rec_ids) h->recs[(size_t)id].host_valid = false;
    RunParams p;
    p.seed = (uint64_t)h->seed;
    p.event_base = h->events;
    p.word_base = (uint64_t)h->word_base;
    p.pad = 0;
    h->events += c->num_events;
    if (reset) h->valid = true;
    return p;
}

// ---- autotuner ---------------------------------------------------------
// Shared-x/z knobs, cached per process by (qubits, shot-words, noise ranges,
// broadcast or not).
struct FrameTuneKey {
    int64_t n, w, nctas;
    bool bcast;
    bool operator<(const FrameTuneKey &o) const {
        if (n != o.n) return n < o.n;
        if (w != o.w) return w < o.w;
        if (nctas != o.nctas) return nctas < o.nctas;
        return bcast < o.bcast;
    }
};
std::mutex g_ftune_mu;
std::map<FrameTuneKey, std::pair<int, int>> g_ftune_cache;

int autotune_frame(ps_circuit *c, double *tune_ms) {
    ps_state *h = c->h;
    const auto t0 = std::chrono::steady_clock::now();
    const FrameTuneKey key{h->n, h->w, c->ftable.nctas, c->ftable.chunks > 0};
    {
        std::lock_guard<std::mutex> lk(g_ftune_mu);
        auto it = g_ftune_cache.find(key);
        if (it != g_ftune_cache.end()) {
            c->opts.frame_warps = it->second.first;
            c->opts.bcast_ctas = it->second.second;
            if (tune_ms) *tune_ms = 0.0;
            return OK;
        }
    }
    set_params_kernel<<<1, 1, 0, h->stream>>>(c->d_params, (uint64_t)h->seed, h->events, (uint64_t)h->word_base);
    PS_CUDA(cudaGetLastError());
    int fw = 8, bc = 1;
    int rc = tune_frame_table(c->ftable, h->stream, c->fstream, c->fev[0], c->fev[1], &fw, &bc, nullptr);
    if (rc != OK) return rc;
    c->opts.frame_warps = fw;
    c->opts.bcast_ctas = bc;
    {
        std::lock_guard<std::mutex> lk(g_ftune_mu);
        g_ftune_cache[key] = {fw, bc};
    }
    if (tune_ms) *tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return OK;
}

struct TuneKey {
    int64_t n, w;
    int nq;
    bool operator<(const TuneKey &o) const {
        return n != o.n ? n < o.n : (w != o.w ? w < o.w : nq < o.nq);
    }
};
struct TuneChoice {
    int rows, words, threads, meas_words;
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneChoice> g_tune_cache;

struct EventTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    EventTimer() {
        cudaEventCreate(&a);
        cudaEventCreate(&b);
    }
    ~EventTimer() {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

int autotune(ps_circuit *c, double *tune_ms) {
    ps_state *h = c->h;
    const auto t0 = std::chrono::steady_clock::now();
    size_t s0 = c->steps.size(), m0 = c->steps.size();
    int nq = 1;
    for (size_t i = 0; i < c->steps.size(); ++i) {
        if (c->steps[i].kind == K_SEGMENT) {
            nq = std::max(nq, (int)c->segs[(size_t)c->steps[i].first].cols.size());
            if (s0 == c->steps.size()) s0 = i;
        }
        if (c->steps[i].kind == K_MEAS && s0 < c->steps.size() && m0 == c->steps.size() && c->steps[i].count > 1) m0 = i;
    }
    if (s0 == c->steps.size()) return OK;
    const TuneKey key{h->n, h->w, nq};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            c->opts.seg_rows = it->second.rows;
            c->opts.seg_words = it->second.words;
            c->opts.seg_threads = it->second.threads;
            c->opts.meas_words = it->second.meas_words;
            if (tune_ms) *tune_ms = 0.0;
            return OK;
        }
    }
    const cudaStream_t st = h->stream;
    set_params_kernel<<<1, 1, 0, st>>>(c->d_params, (uint64_t)h->seed, h->events, (uint64_t)h->word_base);
    PS_CUDA(cudaGetLastError());
    auto prefix = [&](size_t upto) -> int {  // |0...0>, then steps [0, upto)
        int rc = launch_init_zero_on(st, h);
        if (rc == OK) rc = enqueue_steps(c, st, 0, upto);
        return rc;
    };
    EventTimer ev;
    auto time_it = [&](auto &&fn, float *ms) -> int {
        PS_CUDA(cudaEventRecord(ev.a, st));
        int rc = fn();
        if (rc != OK) return rc;
        PS_CUDA(cudaEventRecord(ev.b, st));
        PS_CUDA(cudaEventSynchronize(ev.b));
        PS_CUDA(cudaEventElapsedTime(ms, ev.a, ev.b));
        return OK;
    };
    // Segment tiles: rows x shot-words x threads.
    const SegHost &sg = c->segs[(size_t)c->steps[s0].first];
    const int cand[][3] = {{1, 2, 64}, {1, 4, 128}, {1, 8, 256}, {2, 4, 256}, {1, 16, 256}, {2, 8, 256}, {4, 2, 256}};
    int rc = prefix(s0);
    if (rc == OK && !sg.slots.empty()) rc = launch_noise_sample(st, sg.dev, h->w, c->d_params);
    if (rc != OK) return rc;
    float best = 3.0e38f;
    TuneChoice pick{c->opts.seg_rows, c->opts.seg_words, c->opts.seg_threads, c->opts.meas_words};
    for (const auto &cd : cand) {
        const int rows = cd[0], bw = cd[1], threads = cd[2];
        if (bw > std::max<int64_t>(2, h->w)) continue;
        if (max_seg_smem(c, rows, bw) > kSegSmemMax) continue;
        auto go = [&] {
            return launch_segment(st, h->X, h->Z, h->R, h->n, h->w, sg.dev, rows, bw, threads, c->d_recs);
        };
        float ms = 0.f, ms2 = 0.f;
        if (time_it(go, &ms) != OK || time_it(go, &ms2) != OK) {  // the first launch also warms up
            cudaGetLastError();
            continue;
        }
        ms = std::min(ms, ms2);
        if (ms < best) {
            best = ms;
            pick.rows = rows;
            pick.words = bw;
            pick.threads = threads;
        }
    }
    c->opts.seg_rows = pick.rows;
    c->opts.seg_words = pick.words;
    c->opts.seg_threads = pick.threads;
    // Measurement kernel: shot-words per CTA (1, 2 or 4), on the first two
    // measurement phases (the first one after reset, one mid-circuit).
    if (m0 < c->steps.size()) {
        size_t m1 = c->steps.size();
        for (size_t i = m0 + 1; i < c->steps.size(); ++i)
            if (c->steps[i].kind == K_MEAS && c->steps[i].count > 1) {
                m1 = i;
                break;
            }
        float bestm = 3.0e38f;
        for (int B = 1; B <= 4; B *= 2) {
            if (h->w % B) continue;
            c->opts.meas_words = B;
            float total = 0.f;
            for (int rep = 0; rep < 2; ++rep) {  // the first pass warms up
                float ms0 = 0.f, ms1 = 0.f;
                rc = prefix(m0);
                if (rc != OK) return rc;
                rc = time_it([&] { return enqueue_steps(c, st, m0, m0 + 1); }, &ms0);
                if (rc != OK) return rc;
                if (m1 < c->steps.size()) {
                    rc = enqueue_steps(c, st, m0 + 1, m1);
                    if (rc != OK) return rc;
                    rc = time_it([&] { return enqueue_steps(c, st, m1, m1 + 1); }, &ms1);
                    if (rc != OK) return rc;
                }
                total = ms0 + ms1;
            }
            if (total < bestm) {
                bestm = total;
                pick.meas_words = B;
            }
        }
        c->opts.meas_words = pick.meas_words;
    }
    PS_CUDA(cudaStreamSynchronize(st));
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune_cache[key] = pick;
    }
    if (tune_ms)
        *tune_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return OK;
}

}  // namespace
}  // namespace ps

extern "C" {

ps_status ps_circuit_compile(ps_state *h, const ps_op *ops_in, uint64_t nops, const float *params, uint64_t nparams,
                             const ps_circuit_options *opts, ps_circuit **out) {
    ps_enter(__func__, __LINE__);
    if (!h || !out) return fail(E_ARG, "null handle");
    if (nops && !ops_in) return fail(E_ARG, "null op table");
    *out = nullptr;
    std::vector<ps_op> ops(ops_in, ops_in + nops);
    auto *c = new ps_circuit;
    c->h = h;
    if (opts) c->opts = *opts;
    const bool fused = c->opts.mode == PS_MODE_FUSED;
    auto bail = [&](int rc) {
        const std::string msg = ps_last_error();
        ps_circuit_destroy(c);
        set_error(msg);  // keep the failing step's message
        return rc;
    };
    if (h->signs_only && (!fused || c->opts.per_shot_xz))
        return bail(fail(E_STATE, "a signs-only state runs only the fused shared-x/z plan"));

    // ---- validate ops, assign events / records / thresholds
    std::vector<uint32_t> event_of(ops.size(), 0);
    std::vector<int32_t> rec_of(ops.size(), -1), thr_off(ops.size(), -1);
    std::vector<uint64_t> thr;
    std::map<std::vector<uint64_t>, int32_t> thr_index;
    // the last probabilities of each channel kind and their table: a noise
    // model puts the same ones on every channel, so most channels are a
    // 12- or 60-byte compare
    float last_p[2][15];
    int32_t last_off[2] = {-1, -1};
    uint32_t ev = 0;
    int32_t nrec = 0;
    for (size_t i = 0; i < ops.size(); ++i) {
        const ps_op &o = ops[i];
        auto qok = [&](int32_t q) { return q >= 0 && q < h->n; };
        if (o.code < OP_H || o.code > OP_S_IF) return bail(fail(E_ARG, "op " + std::to_string(i) + ": bad code"));
        if (!qok(o.a)) return bail(fail(E_ARG, "op " + std::to_string(i) + ": qubit out of range"));
        if ((o.code == OP_CX || o.code == OP_CZ || o.code == OP_PAULI2) && (!qok(o.b) || o.b == o.a))
            return bail(fail(E_ARG, "op " + std::to_string(i) + ": bad second qubit"));
        if (o.code == OP_H_IF || o.code == OP_S_IF) {
            if (o.c < 0 || o.c >= nrec) return bail(fail(E_ARG, "op " + std::to_string(i) + ": record not measured yet"));
        }
        if (o.code == OP_M && o.c >= 0 && (uint64_t)o.c >= nparams)
            return bail(fail(E_ARG, "op " + std::to_string(i) + ": bias index out of range"));
        if (o.code == OP_M && o.c >= 0 && !(params[o.c] >= 0.0f && params[o.c] <= 1.0f))
            return bail(fail(E_ARG, "op " + std::to_string(i) + ": bias is not a number in [0, 1]"));
        if (is_channel(o.code)) {
            const int cnt = o.code == OP_PAULI2 ? 15 : 3, kind = o.code == OP_PAULI2 ? 1 : 0;
            if (o.c < 0 || (uint64_t)o.c + cnt > nparams)
                return bail(fail(E_ARG, "op " + std::to_string(i) + ": channel parameters out of range"));
            if (last_off[kind] >= 0 && std::memcmp(last_p[kind], params + o.c, (size_t)cnt * sizeof(float)) == 0) {
                thr_off[i] = last_off[kind];  // checked and tabled already
                event_of[i] = ev++;
                continue;
            }
            if (check_channel_probs(params + o.c, cnt) != OK)
                return bail(fail(E_ARG, "op " + std::to_string(i) + ": " + ps_last_error()));
            uint64_t t[16];
            channel_thresholds(params + o.c, cnt, t);
            // one copy of each distinct table (the same probabilities on
            // every channel of a noise model is the usual case)
            std::vector<uint64_t> key(t, t + cnt + 1);
            auto it = thr_index.find(key);
            if (it == thr_index.end()) {
                it = thr_index.emplace(std::move(key), (int32_t)thr.size()).first;
                thr.insert(thr.end(), t, t + cnt + 1);
            }
            thr_off[i] = it->second;
            std::memcpy(last_p[kind], params + o.c, (size_t)cnt * sizeof(float));
            last_off[kind] = it->second;
        }
        if (is_meas(o.code)) rec_of[i] = nrec++;
        if (is_meas(o.code) || is_channel(o.code)) event_of[i] = ev++;
    }
    c->num_events = ev;
    c->thr_host = thr;

    // ---- records: one contiguous block, so a run's records copy out at once
    c->stats.first_record = h->recs.size();
    {
        std::vector<int64_t> qubits;
        for (size_t i = 0; i < ops.size(); ++i)
            if (is_meas(ops[i].code)) qubits.push_back(ops[i].a);
        int rc = record_block(h, qubits, c->rec_ids, &c->d_res_block, &c->d_det_block);
        if (rc != OK) return bail(rc);
    }
    std::vector<u64 *> rec_ptrs;
    for (int64_t id : c->rec_ids) rec_ptrs.push_back(h->recs[(size_t)id].res);
    if (upload(h, c->owned, rec_ptrs, &c->d_recs) != OK) return bail(E_CUDA);
    if (thr.empty()) thr.push_back(0);
    if (upload(h, c->owned, thr, &c->d_thr) != OK) return bail(E_CUDA);
    {
        void *p = nullptr;
        if (dev_alloc(h, &p, sizeof(RunParams)) != OK) return bail(E_NOMEM);
        c->owned.push_back(p);
        c->d_params = (RunParams *)p;
        if (dev_alloc(h, &p, 4 * (size_t)h->w * sizeof(u64)) != OK) return bail(E_NOMEM);
        c->owned.push_back(p);
        c->d_masks = (u64 *)p;
    }

    // ---- plan (from the cache when this circuit was compiled before)
    const std::string pkey = plan_key(h, c->opts, ops, params, nparams);
    const std::shared_ptr<const PlanCacheEntry> cached = fused ? plan_lookup(pkey) : nullptr;
    std::shared_ptr<PlanCacheEntry> fresh;
    auto add_meas = [&](size_t i, int reset) {
        MeasOp m{};
        m.q = ops[i].a;
        m.reset = reset;
        m.bias = (ops[i].code == OP_M && ops[i].c >= 0) ? params[ops[i].c] : 0.5f;
        m.event = event_of[i];
        m.forced = nullptr;
        const Record &r = h->recs[(size_t)c->rec_ids[(size_t)rec_of[i]]];
        m.res = r.res;
        m.det = r.det;
        c->meas.push_back(m);
        c->meas_op.push_back((int32_t)i);
    };
    size_t max_slots = 0;
    std::map<int32_t, int32_t> ptable;  // plain form: thr offset -> distinct table
    std::vector<uint32_t> psurv;
    if (!fused) {
        for (size_t i = 0; i < ops.size(); ++i) {
            const ps_op &o = ops[i];
            Step s{};
            if (is_meas(o.code)) {
                s.kind = K_MEAS;
                s.first = (int32_t)c->meas.size();
                s.count = 1;
                add_meas(i, o.code == OP_R);
            } else if (is_channel(o.code)) {
                s.kind = K_CHANNEL;
                s.a = o.a;
                s.b = o.code == OP_PAULI2 ? o.b : 0;
                s.count = o.code == OP_PAULI2 ? 15 : 3;
                s.first = thr_off[i];
                s.event = event_of[i];
                auto tt = ptable.find(thr_off[i]);
                if (tt == ptable.end()) {  // survival products and estimate factors of a new table
                    tt = ptable.emplace(thr_off[i], (int32_t)c->pest.size()).first;
                    const uint64_t total = thr[(size_t)(thr_off[i] + s.count - 1)];
                    c->pest.push_back(channel_est_factors(total, s.count));
                    psurv.resize(psurv.size() + 64, 0u);
                    channel_surv_table(total, &psurv[psurv.size() - 64]);
                }
                s.table = tt->second;
            } else {
                s.kind = K_GATE;
                s.code = o.code;
                s.a = o.a;
                s.b = (o.code == OP_CX || o.code == OP_CZ) ? o.b : 0;
                s.rec = (o.code == OP_H_IF || o.code == OP_S_IF) ? o.c : -1;
            }
            c->steps.push_back(s);
        }
    } else if (cached) {
        c->steps = cached->steps;
        c->segs = cached->segs;
        c->meas = cached->meas;
        c->meas_op = cached->meas_op;
        for (size_t m = 0; m < c->meas.size(); ++m) {  // this compile's records
            const Record &r = h->recs[(size_t)c->rec_ids[(size_t)rec_of[(size_t)c->meas_op[m]]]];
            c->meas[m].res = r.res;
            c->meas[m].det = r.det;
        }
        for (const SegHost &sg : c->segs) max_slots = std::max(max_slots, sg.slots.size());
    } else {
        std::vector<std::pair<int64_t, int32_t>> pending;  // deferred reset X: (qubit, record)
        size_t i = 0;
        while (i < ops.size()) {
            size_t j = i;
            if (is_meas(ops[i].code)) {
                while (j < ops.size() && is_meas(ops[j].code)) ++j;
                const bool more_segments = j < ops.size();
                Step s{};
                s.kind = K_MEAS;
                s.first = (int32_t)c->meas.size();
                s.count = (int32_t)(j - i);
                for (size_t k = i; k < j; ++k) {
                    bool later_same = false;
                    for (size_t t = k + 1; t < j; ++t) later_same |= ops[t].a == ops[k].a;
                    const bool defer = ops[k].code == OP_R && h->valid && more_segments && !later_same;
                    add_meas(k, ops[k].code == OP_R && !defer);
                    if (defer) pending.emplace_back(ops[k].a, rec_of[k]);
                }
                c->steps.push_back(s);
            } else {
                while (j < ops.size() && !is_meas(ops[j].code)) ++j;
                SegHost seg;
                build_segment(c, ops, i, j, event_of, rec_of, thr_off, pending, seg);
                pending.clear();
                max_slots = std::max(max_slots, seg.slots.size());
                Step s{};
                s.kind = K_SEGMENT;
                s.first = (int32_t)c->segs.size();
                c->segs.push_back(std::move(seg));
                c->steps.push_back(s);
            }
            i = j;
        }
        fresh = std::make_shared<PlanCacheEntry>();
        fresh->steps = c->steps;
        fresh->segs = c->segs;
        fresh->meas = c->meas;
        for (MeasOp &m : fresh->meas) m.res = m.det = nullptr;
        fresh->meas_op = c->meas_op;
    }
    if (!fused) {
        if (psurv.empty()) psurv.assign(64, 0u);
        if (upload(h, c->owned, psurv, &c->d_psurv) != OK) return bail(E_CUDA);
    }
    pick_tile(c);
    for (const SegHost &sg : c->segs) {  // algorithmic bytes of the per-shot segments (host data)
        const double W = (double)h->W, B8 = (double)h->S / 8.0;
        c->stats.segment_bytes += 2.0 * (2.0 * (double)sg.cols.size() + 1.0) * W * B8;
    }
    c->max_slots = max_slots;
    if (upload(h, c->owned, c->meas, &c->d_meas) != OK) return bail(E_CUDA);

    // ---- shared-x/z plan of runs from |0...0> (no per-shot conditional gates)
    if (fused && c->opts.per_shot_xz == 0 && h->n > 0 && frame_smem_bytes(h->n) <= kSegSmemMax) {
        bool ok = true;
        for (const ps_op &o : ops) ok &= o.code != OP_H_IF && o.code != OP_S_IF;
        if (ok && cached && cached->has_frame) {
            c->fprog = cached->fprog;
        } else if (ok) {
            FrameBuilder fb(h->n);
            for (const Step &s : c->steps) {
                if (s.kind == K_SEGMENT) {
                    const SegHost &sg = c->segs[(size_t)s.first];
                    std::map<size_t, uint32_t> slot_of;
                    for (size_t k = 0; k < sg.slot_op.size(); ++k) slot_of[(size_t)sg.slot_op[k]] = (uint32_t)k;
                    fb.begin_segment(s.first, (uint32_t)sg.slots.size(), sg.op1 - sg.op0);
                    for (size_t i = sg.op0; i < sg.op1; ++i) {
                        const ps_op &o = ops[i];
                        if (is_channel(o.code))
                            fb.channel(o.a, o.code == OP_PAULI2 ? o.b : -1, slot_of[i]);
                        else
                            fb.gate(o.code, o.a, o.b);
                    }
                    fb.end_segment();
                } else if (s.kind == K_MEAS) {
                    for (int32_t m = s.first; m < s.first + s.count; ++m) {
                        const ps_op &o = ops[(size_t)c->meas_op[(size_t)m]];
                        fb.measure(o.a, m, o.code == OP_R);
                    }
                }
            }
            fb.finish();
            // F_LINEAR scratch: what shared memory leaves beside the signs
            // and up to n random outcomes of a launch
            const size_t fixed = frame_smem_bytes(h->n) + (size_t)h->n * sizeof(u64) + 16;
            fb.linearize(fixed < kSegSmemMax ? (uint32_t)std::min<size_t>((kSegSmemMax - fixed) / sizeof(u64), 1u << 20)
                                             : 0u);
            c->fprog = std::move(fb.prog);
            c->fprog.tab.insert(c->fprog.tab.end(), 4, 0u);  // padding: staged ranges round up to 16 bytes
            if (c->fprog.slot_off.empty()) c->fprog.slot_off.push_back(0);
            if (c->fprog.rand_meas.empty()) c->fprog.rand_meas.push_back(0);
            if (fresh) {
                fresh->has_frame = true;
                fresh->fprog = c->fprog;
            }
        }
        if (ok) {
            if (upload(h, c->owned, c->fprog.ops, &c->d_fops) || upload(h, c->owned, c->fprog.tab, &c->d_ftab) ||
                upload(h, c->owned, c->fprog.xz, &c->d_fxz) ||
                upload(h, c->owned, c->fprog.rand_meas, &c->d_frand))
                return bail(E_CUDA);
            FrameJobDev job{};
            std::vector<FrameRangeDev> ranges;
            std::vector<FrameSlotDev> fslots;
            std::vector<uint32_t> fs64, fev;
            std::vector<int32_t> nvr;
            std::vector<FrameChanTab> ctabs;
            std::vector<uint32_t> surv;
            const int jrc = frame_job_ranges(c, job, ranges, fslots, fs64, fev, nvr, ctabs, surv);
            if (jrc == E_ARG) {
                set_error("");  // the program does not fit the one-launch kernel: the per-shot plan runs
                ok = false;
            } else if (jrc != OK) {
                return bail(jrc);
            }
            if (ok) {  // the job table of one job
                FrameRangeDev *dr = nullptr;
                FrameSlotDev *dsl = nullptr;
                FrameChanTab *dct = nullptr;
                uint32_t *dsv = nullptr, *ds64 = nullptr, *dev = nullptr;
                int32_t *dnvr = nullptr;
                if (upload(h, c->owned, ranges, &dr) || upload(h, c->owned, fslots, &dsl) ||
                    upload(h, c->owned, fs64, &ds64) || upload(h, c->owned, fev, &dev) || upload(h, c->owned, ctabs, &dct) ||
                    upload(h, c->owned, surv, &dsv) || upload(h, c->owned, nvr, &dnvr))
                    return bail(E_CUDA);
                job.nv_range = dnvr;
                if (job.nnv > 0) {  // the noise vectors: [nnv][w][Wp] words
                    void *pn = nullptr;
                    const size_t nb = (size_t)job.nnv * (size_t)h->w * (size_t)frame_wp(h->n) * sizeof(u64);
                    if (dev_alloc(h, &pn, nb) != OK) return bail(fail(E_NOMEM, "device allocation of noise vectors failed"));
                    c->owned.push_back(pn);
                    job.nvec = static_cast<u64 *>(pn);
                }
                job.ranges = dr;
                job.slot = dsl;
                job.slot_s64 = ds64;
                job.slot_event = dev;
                {  // the error word (offset 0) and the broadcast's counters (offsets 16, 24)
                    void *pe = nullptr;
                    if (dev_alloc(h, &pe, 32) != OK) return bail(E_NOMEM);
                    c->owned.push_back(pe);
                    c->d_ferr = static_cast<int32_t *>(pe);
                    if (cudaMemsetAsync(pe, 0, 32, h->stream) != cudaSuccess)
                        return bail(cuda_fail(cudaGetLastError(), "cudaMemsetAsync"));
                    job.err = c->d_ferr;
                    c->ftable.bctr = reinterpret_cast<unsigned long long *>(static_cast<char *>(pe) + 16);
                }
                job.ctab = dct;
                job.surv = dsv;
                BroadcastJobDev bj{h->X, h->Z, c->d_fxz, h->n, h->w, c->fprog.nw64};
                const std::vector<FrameJobDev> jobs{job};
                const std::vector<BroadcastJobDev> bjobs{bj};
                const std::vector<int64_t> cta0{0, h->w}, chunk0{0, broadcast_chunks(h->n, h->w)},
                    ncta0{0, (int64_t)job.nnv * h->w};
                FrameJobDev *dj = nullptr;
                BroadcastJobDev *db = nullptr;
                int64_t *dc = nullptr, *dk = nullptr, *dn = nullptr;
                if (upload(h, c->owned, jobs, &dj) || upload(h, c->owned, bjobs, &db) ||
                    upload(h, c->owned, cta0, &dc) || upload(h, c->owned, chunk0, &dk) || upload(h, c->owned, ncta0, &dn))
                    return bail(E_CUDA);
                c->ftable.jobs = dj;
                c->ftable.bjobs = db;
                c->ftable.cta0 = dc;
                c->ftable.ncta0 = dn;
                c->ftable.chunk0 = dk;
                c->ftable.njobs = 1;
                c->ftable.ctas = h->w;
                c->ftable.nctas = ncta0[1];
                c->ftable.chunks = h->signs_only ? 0 : chunk0[1];  // signs only: no x / z to write
                c->ftable.smem = frame_job_smem(job);
                c->ftable.nsmem = job.nnv > 0 ? noise_job_smem(job) : 0;
                c->fjob = job;
                c->fbjob = bj;
                if (!h->signs_only && cudaStreamCreateWithFlags(&c->fstream, cudaStreamNonBlocking) != cudaSuccess)
                    return bail(cuda_fail(cudaGetLastError(), "cudaStreamCreate"));
                for (cudaEvent_t &e : c->fev)
                    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
                        return bail(cuda_fail(cudaGetLastError(), "cudaEventCreate"));
                c->frame_ok = true;
            }
        }
    }
    if (h->signs_only && !c->frame_ok)
        return bail(fail(E_STATE, "the circuit needs per-shot tableaux, which a signs-only state does not hold"));
    if (fused && !c->frame_ok) {  // every run takes the per-shot plan
        int rc = ensure_segments_dev(c);
        if (rc != OK) return bail(rc);
    }

    // ---- stats
    ps_circuit_stats &st = c->stats;
    st.num_ops = ops.size();
    for (auto &o : ops) {
        if (o.code <= OP_R) st.num_gates++;
        if (is_meas(o.code)) st.num_measurements++;
        if (is_channel(o.code)) st.num_channels++;
    }
    st.num_events = c->num_events;
    for (auto &s : c->steps) {
        if (s.kind == K_SEGMENT) {
            st.num_segments++;
            st.launches_per_run += c->segs[(size_t)s.first].slots.empty() ? 1 : 3;
        } else if (s.kind == K_MEAS) {
            st.num_measure_phases++;
            st.launches_per_run += 1;
        } else if (s.kind == K_CHANNEL) {
            st.launches_per_run += 1;
        } else {
            st.launches_per_run += 1;
        }
    }
    st.launches_per_run += 1;  // run-parameter update
    if (c->frame_ok) {  // runs from |0...0>: the parameters, the sign kernel, the broadcast
        st.shared_xz = 1;
        // parameters, noise vectors (when there are channels), signs, broadcast (unless signs only)
        st.launches_per_run = 2 + (c->ftable.nctas > 0 ? 1 : 0) + (c->ftable.chunks > 0 ? 1 : 0);
        st.frame_warps = c->opts.frame_warps > 0 ? c->opts.frame_warps : 8;
        st.bcast_ctas = c->opts.bcast_ctas > 0 ? c->opts.bcast_ctas : 1;
    }
    st.seg_rows = c->opts.seg_rows;
    st.seg_words = c->opts.seg_words;
    st.seg_threads = c->opts.seg_threads;
    st.meas_words = c->opts.meas_words;
    for (const SegHost &sg : c->segs) st.resident_segments += sg.res_slots > 0 ? 1 : 0;

    // The tables above were copied on the state's stream; runs may be
    // launched on other streams (graphs, batches).
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(cuda_fail(cudaGetLastError(), "upload"));

    // ---- graph capture
    if (c->opts.use_graph) {
        int rc = capture_graphs(c);
        if (rc != OK) return bail(rc);
    }
    if (fresh) plan_store(pkey, fresh);
    *out = c;
    return OK;
}

ps_status ps_compile_cache_stats(uint64_t *hits, uint64_t *misses, uint64_t *entries) {
    ps_enter(__func__, __LINE__);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    if (hits) *hits = g_plan_hits;
    if (misses) *misses = g_plan_misses;
    if (entries) *entries = g_plan.size();
    return OK;
}

ps_status ps_compile_cache_clear(void) {
    ps_enter(__func__, __LINE__);
    std::lock_guard<std::mutex> lk(g_plan_mu);
    g_plan.clear();
    g_plan_order.clear();
    g_plan_hits = g_plan_misses = 0;
    return OK;
}

ps_status ps_circuit_set_forced(ps_circuit *c, const uint8_t *forced_all) {
    ps_enter(__func__, __LINE__);
    if (!c) return fail(E_ARG, "null circuit");
    ps_state *h = c->h;
    const size_t nm = c->meas.size();
    if (forced_all && nm) {
        if (!c->d_forced) {
            void *p = nullptr;
            if (dev_alloc(h, &p, nm * (size_t)h->w * sizeof(u64)) != OK)
                return fail(E_NOMEM, "device allocation of forced draws failed");
            c->d_forced = (u64 *)p;
        }
        std::vector<u64> buf(nm * (size_t)h->w, 0ull);
        const size_t nb = (size_t)(h->S + 7) / 8;
        for (size_t k = 0; k < nm; ++k) {
            std::memcpy(&buf[k * (size_t)h->w], forced_all + k * nb, nb);
            if (h->S % 8) reinterpret_cast<uint8_t *>(&buf[k * (size_t)h->w])[nb - 1] &= (uint8_t)((1u << (h->S % 8)) - 1u);
        }
        PS_CUDA(cudaMemcpy(c->d_forced, buf.data(), buf.size() * sizeof(u64), cudaMemcpyHostToDevice));
    }
    // Measurement k of the circuit (program order) is meas[] entry k.
    std::vector<MeasOp> m = c->meas;
    for (size_t k = 0; k < nm; ++k) m[k].forced = forced_all ? c->d_forced + k * (size_t)h->w : nullptr;
    PS_CUDA(cudaStreamSynchronize(h->stream));
    PS_CUDA(cudaMemcpy(c->d_meas, m.data(), nm * sizeof(MeasOp), cudaMemcpyHostToDevice));
    c->meas = m;
    return OK;
}

ps_status ps_circuit_run(ps_circuit *c, int reset_state) {
    ps_enter(__func__, __LINE__);
    if (!c) return fail(E_ARG, "null circuit");
    ps_state *h = c->h;
    if (h->signs_only && !reset_state) return fail(E_STATE, "a signs-only state runs only from |0...0>");
    NvtxRange range("ps circuit run");
    if (c->copy_pending) PS_CUDA(cudaStreamWaitEvent(h->stream, c->ev_copied, 0));  // it rewrites those records
    const RunParams p = begin_run(c, reset_state != 0);
    set_params_kernel<<<1, 1, 0, h->stream>>>(c->d_params, p.seed, p.event_base, p.word_base);
    PS_CUDA(cudaGetLastError());
    if (!reset_state && c->opts.use_graph && !c->exec[0] && c->frame_ok && !h->signs_only &&
        c->seg_dev_status < 0) {
        // the first run without reset of a shared-x/z circuit: build and capture its per-shot plan
        int rc = ensure_segments_dev(c);
        if (rc == OK) rc = capture_graph(c, 0);
        if (rc != OK) return rc;
    }
    if (c->exec[reset_state ? 1 : 0]) {
        PS_CUDA(cudaGraphLaunch(c->exec[reset_state ? 1 : 0], h->stream));
        return OK;
    }
    return enqueue_plan(c, h->stream, reset_state != 0);
}

ps_status ps_circuit_profile(ps_circuit *c, int reset_state, ps_circuit_profile_t *out) {
    ps_enter(__func__, __LINE__);
    if (!c || !out) return fail(E_ARG, "null argument");
    ps_state *h = c->h;
    std::memset(out, 0, sizeof(*out));
    const RunParams p = begin_run(c, reset_state != 0);
    set_params_kernel<<<1, 1, 0, h->stream>>>(c->d_params, p.seed, p.event_base, p.word_base);
    PS_CUDA(cudaGetLastError());
    Profiler prof;
    prof.st = h->stream;
    int rc = enqueue_plan(c, h->stream, reset_state != 0, &prof);
    if (rc != OK) return rc;
    PS_CUDA(cudaStreamSynchronize(h->stream));
    for (auto &m : prof.marks) {
        float ms = 0.f;
        PS_CUDA(cudaEventElapsedTime(&ms, m.second.first, m.second.second));
        out->ms[m.first] += ms;
        out->launches[m.first] += 1;
    }
    return OK;
}

ps_status ps_circuit_measure_stats(ps_circuit *c, int reset_state, int32_t *random_branch, int32_t *rows) {
    ps_enter(__func__, __LINE__);
    if (!c || !random_branch || !rows) return fail(E_ARG, "null argument");
    ps_state *h = c->h;
    if (h->signs_only) return fail(E_STATE, "measurement statistics need per-shot tableaux");
    const size_t nm = c->meas.size();
    if (nm == 0) return OK;
    int32_t *d = nullptr;
    PS_CUDA(cudaMalloc(&d, nm * 2 * sizeof(int32_t)));
    std::vector<MeasOp> m = c->meas;
    for (size_t k = 0; k < nm; ++k) m[k].kstat = d + 2 * k;
    PS_CUDA(cudaStreamSynchronize(h->stream));
    PS_CUDA(cudaMemcpy(c->d_meas, m.data(), nm * sizeof(MeasOp), cudaMemcpyHostToDevice));
    const RunParams p = begin_run(c, reset_state != 0);
    set_params_kernel<<<1, 1, 0, h->stream>>>(c->d_params, p.seed, p.event_base, p.word_base);
    c->force_per_shot = true;  // the statistics come from the per-shot measurement kernel
    int rc = enqueue_plan(c, h->stream, reset_state != 0);
    c->force_per_shot = false;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    std::vector<int32_t> host(nm * 2);
    if (rc == OK && e == cudaSuccess) e = cudaMemcpy(host.data(), d, nm * 2 * sizeof(int32_t), cudaMemcpyDeviceToHost);
    cudaMemcpy(c->d_meas, c->meas.data(), nm * sizeof(MeasOp), cudaMemcpyHostToDevice);
    cudaFree(d);
    if (rc != OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "measure stats");
    for (size_t k = 0; k < nm; ++k) {
        random_branch[k] = host[2 * k];
        rows[k] = host[2 * k + 1];
    }
    return OK;
}

ps_status ps_circuit_copy_records(ps_circuit *c, uint64_t *results, uint64_t *determined, uint64_t *words) {
    ps_enter(__func__, __LINE__);
    if (!c) return fail(E_ARG, "null circuit");
    ps_state *h = c->h;
    const size_t bytes = c->rec_ids.size() * (size_t)h->w * sizeof(u64);
    if (words) *words = (uint64_t)h->w;
    if (results && bytes)
        PS_CUDA(cudaMemcpyAsync(results, c->d_res_block, bytes, cudaMemcpyDeviceToHost, h->stream));
    if (determined && bytes)
        PS_CUDA(cudaMemcpyAsync(determined, c->d_det_block, bytes, cudaMemcpyDeviceToHost, h->stream));
    int32_t err = 0;  // the sign kernel's error word (shared-x/z runs)
    if (c->d_ferr) PS_CUDA(cudaMemcpyAsync(&err, c->d_ferr, sizeof err, cudaMemcpyDeviceToHost, h->stream));
    PS_CUDA(cudaStreamSynchronize(h->stream));
    if (err) return fail(E_TIMEOUT, "a copy of the sign program did not arrive in time; the run's records are void");
    return OK;
}

ps_status ps_circuit_copy_records_async(ps_circuit *c, uint64_t *results, uint64_t *determined, void *copy_stream) {
    ps_enter(__func__, __LINE__);
    if (!c) return fail(E_ARG, "null circuit");
    ps_state *h = c->h;
    if (!c->ev_ran) {
        PS_CUDA(cudaEventCreateWithFlags(&c->ev_ran, cudaEventDisableTiming));
        PS_CUDA(cudaEventCreateWithFlags(&c->ev_copied, cudaEventDisableTiming));
        PS_CUDA(cudaMallocHost(&c->h_err, sizeof(int32_t)));
    }
    cudaStream_t cs = static_cast<cudaStream_t>(copy_stream);
    if (!cs) {
        if (!c->cstream_own) PS_CUDA(cudaStreamCreateWithFlags(&c->cstream_own, cudaStreamNonBlocking));
        cs = c->cstream_own;
    }
    const size_t bytes = c->rec_ids.size() * (size_t)h->w * sizeof(u64);
    *c->h_err = 0;
    PS_CUDA(cudaEventRecord(c->ev_ran, h->stream));
    PS_CUDA(cudaStreamWaitEvent(cs, c->ev_ran, 0));
    if (results && bytes) PS_CUDA(cudaMemcpyAsync(results, c->d_res_block, bytes, cudaMemcpyDeviceToHost, cs));
    if (determined && bytes) PS_CUDA(cudaMemcpyAsync(determined, c->d_det_block, bytes, cudaMemcpyDeviceToHost, cs));
    if (c->d_ferr) PS_CUDA(cudaMemcpyAsync(c->h_err, c->d_ferr, sizeof(int32_t), cudaMemcpyDeviceToHost, cs));
    PS_CUDA(cudaEventRecord(c->ev_copied, cs));
    c->copy_pending = true;
    return OK;
}

ps_status ps_circuit_wait_records(ps_circuit *c) {
    ps_enter(__func__, __LINE__);
    if (!c) return fail(E_ARG, "null circuit");
    if (!c->copy_pending) return OK;
    PS_CUDA(cudaEventSynchronize(c->ev_copied));
    c->copy_pending = false;
    if (*c->h_err) return fail(E_TIMEOUT, "a copy of the sign program did not arrive in time; the run's records are void");
    return OK;
}

ps_status ps_circuit_autotune(ps_circuit *c, ps_circuit_options *chosen, double *tune_ms) {
    ps_enter(__func__, __LINE__);
    if (!c) return fail(E_ARG, "null circuit");
    if (tune_ms) *tune_ms = 0.0;
    if (c->opts.mode != PS_MODE_FUSED) {
        if (chosen) *chosen = c->opts;
        return OK;
    }
    if (c->frame_ok) {  // the shared-x/z kernels that runs from |0...0> use
        double ms = 0.0;
        int rc = autotune_frame(c, &ms);
        if (rc != OK) return rc;
        if (tune_ms) *tune_ms += ms;
        c->stats.frame_warps = c->opts.frame_warps;
        c->stats.bcast_ctas = c->opts.bcast_ctas;
    }
    // the per-shot plan's tiles, when its runs take that plan (or it is built already)
    if (!c->h->signs_only && (!c->frame_ok || c->seg_dev_ready)) {
        double ms = 0.0;
        int rc = autotune(c, &ms);
        if (rc != OK) return rc;
        if (tune_ms) *tune_ms += ms;
        c->stats.seg_rows = c->opts.seg_rows;
        c->stats.seg_words = c->opts.seg_words;
        c->stats.seg_threads = c->opts.seg_threads;
        c->stats.meas_words = c->opts.meas_words;
    }
    if (c->opts.use_graph) {
        int rc = capture_graphs(c);
        if (rc != OK) return rc;
    }
    if (chosen) *chosen = c->opts;
    return OK;
}

ps_status ps_circuit_detectors(ps_circuit *c, const uint32_t *idx, const uint64_t *off, uint64_t ndet,
                               uint64_t *out) {
    ps_enter(__func__, __LINE__);
    if (!c || (ndet && (!idx || !off || !out))) return fail(E_ARG, "null argument");
    if (ndet == 0) return OK;
    ps_state *h = c->h;
    const uint64_t nm = c->rec_ids.size();
    if (off[0] != 0) return fail(E_ARG, "detector offsets must start at 0");
    for (uint64_t d = 0; d < ndet; ++d)
        if (off[d + 1] < off[d]) return fail(E_ARG, "detector offsets must not decrease");
    const uint64_t nidx = off[ndet];
    for (uint64_t j = 0; j < nidx; ++j)
        if (idx[j] >= nm) return fail(E_RANGE, "detector refers to measurement " + std::to_string(idx[j]) +
                                                   " of a circuit with " + std::to_string(nm));
    void *d_idx = nullptr, *d_off = nullptr, *d_out = nullptr;
    const size_t out_bytes = (size_t)ndet * (size_t)h->w * sizeof(u64);
    int rc = dev_alloc(h, &d_idx, std::max<uint64_t>(1, nidx) * sizeof(uint32_t));
    if (rc == OK) rc = dev_alloc(h, &d_off, (ndet + 1) * sizeof(uint64_t));
    if (rc == OK) rc = dev_alloc(h, &d_out, out_bytes);
    auto cleanup = [&] {
        cudaStreamSynchronize(h->stream);
        dev_free(h, d_idx);
        dev_free(h, d_off);
        dev_free(h, d_out);
    };
    if (rc != OK) {
        cleanup();
        return rc;
    }
    cudaError_t e = cudaSuccess;
    if (nidx) e = cudaMemcpyAsync(d_idx, idx, nidx * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_off, off, (ndet + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) {
        const int64_t work = (int64_t)ndet * h->w;
        const int blocks = (int)std::min<int64_t>((work + 255) / 256, 152 * 16);
        detector_kernel<<<blocks, 256, 0, h->stream>>>(c->d_res_block, h->w, (const uint32_t *)d_idx,
                                                        (const uint64_t *)d_off, (int64_t)ndet, (u64 *)d_out);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, out_bytes, cudaMemcpyDeviceToHost, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(e, "detectors");
    return OK;
}

ps_status ps_circuit_get_stats(const ps_circuit *c, ps_circuit_stats *out) {
    ps_enter(__func__, __LINE__);
    if (!c || !out) return fail(E_ARG, "null argument");
    *out = c->stats;
    return OK;
}

ps_status ps_circuit_destroy(ps_circuit *c) {
    ps_enter(__func__, __LINE__);
    if (!c) return OK;
    if (c->h && c->h->stream) cudaStreamSynchronize(c->h->stream);
    for (int k = 0; k < 2; ++k) {
        if (c->exec[k]) cudaGraphExecDestroy(c->exec[k]);
        if (c->graph[k]) cudaGraphDestroy(c->graph[k]);
    }
    if (c->fstream) {
        cudaStreamSynchronize(c->fstream);
        cudaStreamDestroy(c->fstream);
    }
    for (cudaEvent_t e : c->fev)
        if (e) cudaEventDestroy(e);
    if (c->ev_copied) cudaEventSynchronize(c->ev_copied);
    if (c->cstream_own) cudaStreamDestroy(c->cstream_own);
    if (c->ev_ran) cudaEventDestroy(c->ev_ran);
    if (c->ev_copied) cudaEventDestroy(c->ev_copied);
    if (c->h_err) cudaFreeHost(c->h_err);
    for (void *p : c->owned) dev_free(c->h, p);
    dev_free(c->h, c->d_forced);
    delete c;
    return OK;
}

}  // extern "C"

namespace ps {
int circuit_enqueue(ps_circuit *c, cudaStream_t st, bool reset) { return enqueue_plan(c, st, reset); }
int frame_table_enqueue(const FrameTable &t, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                        int warps, int bctas) {
    return enqueue_frame_table(t, st, side, fork, join, warps, bctas, nullptr);
}
int frame_table_tune(const FrameTable &t, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                     int *warps, int *bctas, double *best_ms) {
    return tune_frame_table(t, st, side, fork, join, warps, bctas, best_ms);
}
bool circuit_frame_job(const ps_circuit *c, FrameJobDev *job, BroadcastJobDev *bjob) {
    if (!c->frame_ok || c->force_per_shot) return false;
    *job = c->fjob;
    *bjob = c->fbjob;
    return true;
}
RunParams circuit_current_params(const ps_circuit *c) {
    RunParams p;
    p.seed = (uint64_t)c->h->seed;
    p.event_base = c->h->events;
    p.word_base = (uint64_t)c->h->word_base;
    p.pad = 0;
    return p;
}
RunParams circuit_begin_run(ps_circuit *c, bool reset) { return begin_run(c, reset); }
RunParams *circuit_params_dev(ps_circuit *c) { return c->d_params; }
ps_state *circuit_state(ps_circuit *c) { return c->h; }
}  // namespace ps
