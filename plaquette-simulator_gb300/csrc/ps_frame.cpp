// ps_frame.cpp -- host side of shared-x/z runs: the x / z simulation of one
// tableau and the sign program it emits (see ps_frame.h).
#include "ps_frame.h"

#include <algorithm>

#include "../../include/plaquette_gpu.h"

namespace ps {

FrameBuilder::FrameBuilder(int64_t n) : n_(n), W_(2 * n + 1), nw_((n + 63) / 64), ww_((2 * n + 1 + 63) / 64) {
    x_.assign((size_t)(W_ * nw_), 0ull);
    z_.assign((size_t)(W_ * nw_), 0ull);
    fb_.assign((size_t)ww_, 0ull);
    for (int64_t i = 0; i < n_; ++i) {  // |0...0>: destabilizer X_i, stabilizer Z_i (CliffordState.hpp:66-71)
        flip(x_, i, i);
        flip(z_, i + n_, i);
    }
    // and r(i) = [i == 2n] (MiscFunctors.hpp:8-28): the device starts every
    // sign at 0, so the scratch row's 1 is a pending flip
    fset(2 * n_, true);
    prog.nw64 = nw_;
    flipped_.assign((size_t)W_, 0);
    open_range();
}

void FrameBuilder::to_col() {
    if (col_) return;
    if (colok_) {  // the copy is exact but for the scratch row
        const int64_t s = 2 * n_;
        const uint64_t m = 1ull << (s & 63);
        for (int64_t q = 0; q < n_; ++q) {
            uint64_t &xw = xc_[(size_t)(q * ww_ + (s >> 6))], &zw = zc_[(size_t)(q * ww_ + (s >> 6))];
            xw = bit(x_, s, q) ? (xw | m) : (xw & ~m);
            zw = bit(z_, s, q) ? (zw | m) : (zw & ~m);
        }
        col_ = true;
        return;
    }
    xc_.assign((size_t)(n_ * ww_), 0ull);
    zc_.assign((size_t)(n_ * ww_), 0ull);
    for (int64_t i = 0; i < W_; ++i)
        for (int64_t t = 0; t < nw_; ++t) {
            for (uint64_t v = x_[(size_t)(i * nw_ + t)]; v; v &= v - 1)
                xc_[(size_t)((64 * t + __builtin_ctzll(v)) * ww_ + (i >> 6))] |= 1ull << (i & 63);
            for (uint64_t v = z_[(size_t)(i * nw_ + t)]; v; v &= v - 1)
                zc_[(size_t)((64 * t + __builtin_ctzll(v)) * ww_ + (i >> 6))] |= 1ull << (i & 63);
        }
    col_ = true;
    colok_ = true;
}

void FrameBuilder::to_row() {
    if (!col_) return;
    std::fill(x_.begin(), x_.end(), 0ull);
    std::fill(z_.begin(), z_.end(), 0ull);
    for (int64_t q = 0; q < n_; ++q)
        for (int64_t t = 0; t < ww_; ++t) {
            for (uint64_t v = xc_[(size_t)(q * ww_ + t)]; v; v &= v - 1)
                x_[(size_t)((64 * t + __builtin_ctzll(v)) * nw_ + (q >> 6))] |= 1ull << (q & 63);
            for (uint64_t v = zc_[(size_t)(q * ww_ + t)]; v; v &= v - 1)
                z_[(size_t)((64 * t + __builtin_ctzll(v)) * nw_ + (q >> 6))] |= 1ull << (q & 63);
        }
    col_ = false;
    colok_ = true;
}

namespace {
// Rows [lo, hi) of a column-major bit column: the first set one (hi if
// none), and each set one in increasing order.
int64_t first_set(const uint64_t *col, int64_t lo, int64_t hi) {
    for (int64_t t = lo >> 6; (t << 6) < hi; ++t) {
        uint64_t v = col[t];
        if ((t << 6) < lo) v &= ~0ull << (lo & 63);
        if (v) {
            const int64_t i = (t << 6) + __builtin_ctzll(v);
            return i < hi ? i : hi;
        }
    }
    return hi;
}

template <class F>
void each_set(const uint64_t *col, int64_t lo, int64_t hi, F &&f) {
    for (int64_t t = lo >> 6; (t << 6) < hi; ++t) {
        uint64_t v = col[t];
        if ((t << 6) < lo) v &= ~0ull << (lo & 63);
        for (; v; v &= v - 1) {
            const int64_t i = (t << 6) + __builtin_ctzll(v);
            if (i >= hi) return;
            f(i);
        }
    }
}
}  // namespace

void FrameBuilder::push_op(const FrameOp &op) {
    prog.ops.push_back(op);
    op_tab_end_.push_back((uint32_t)prog.tab.size());
    prog.launches.back().op1 = (uint32_t)prog.ops.size();
}

void FrameBuilder::flush_window() {
    if (window_.empty()) return;
    FrameOp op{};
    op.kind = F_WINDOW;
    op.off = (uint32_t)prog.tab.size();
    op.len = (uint32_t)window_.size();
    const uint32_t s = (uint32_t)(2 * n_), zero_row = (uint32_t)W_;
    for (size_t j = 0; j < window_.size(); ++j) {
        DetRecord &r = window_[j];
        if (j + 1 < window_.size())  // the last measurement of the window overwrites the scratch row
            r.rs.erase(std::remove(r.rs.begin(), r.rs.end(), s), r.rs.end());
        prog.tab.push_back((uint32_t)r.meas);
        prog.tab.push_back(r.c | (uint32_t)r.rd.size() << 1 | (uint32_t)r.rs.size() << 4);
        for (uint32_t t = 0; t < kWinRows; ++t) prog.tab.push_back(t < r.rd.size() ? r.rd[t] : zero_row);
        for (uint32_t t = 0; t < kWinRows; ++t) prog.tab.push_back(t < r.rs.size() ? r.rs[t] : (uint32_t)W_ + 1 + t);
    }
    push_op(op);
    window_.clear();
    ++stamp_;
}

void FrameBuilder::open_range() {
    prog.launches.push_back(
        {-1, (uint32_t)prog.ops.size(), (uint32_t)prog.ops.size(), 0, 0, (uint32_t)prog.rand_meas.size(), 0});
}

// The gate functors of GateFunctors.hpp over all W rows (scratch included,
// CliffordState.hpp:381-386), 64 rows per word: x / z updated here, the sign
// term folded into f.
void FrameBuilder::gate(int32_t code, int64_t a, int64_t b) {
    if (!seg_col_) {  // a short segment: row by row on the row-major bits
        to_row();
        colok_ = false;
        for (int64_t i = 0; i < W_; ++i) {
            const int xa = bit(x_, i, a), za = bit(z_, i, a);
            int fl = 0;
            switch (code) {
            case PS_OP_H:
                fl = xa & za;
                if (xa != za) {
                    flip(x_, i, a);
                    flip(z_, i, a);
                }
                break;
            case PS_OP_S:
                fl = xa & za;
                if (xa) flip(z_, i, a);
                break;
            case PS_OP_X: fl = za; break;
            case PS_OP_Y: fl = za ^ xa; break;
            case PS_OP_Z: fl = xa; break;
            case PS_OP_CX: {
                const int xt = bit(x_, i, b), zt = bit(z_, i, b);
                fl = xa & zt & (xt ^ za ^ 1);
                if (xa) flip(x_, i, b);
                if (zt) flip(z_, i, a);
                break;
            }
            case PS_OP_CZ: {
                const int xt = bit(x_, i, b), zt = bit(z_, i, b);
                fl = xa & xt & (zt ^ za);
                if (xa) flip(z_, i, b);
                if (xt) flip(z_, i, a);
                break;
            }
            default: break;
            }
            if (fl) fset(i, !fget(i));
        }
        return;
    }
    to_col();
    uint64_t *xa = &xc_[(size_t)(a * ww_)], *za = &zc_[(size_t)(a * ww_)];
    uint64_t *xb = b >= 0 ? &xc_[(size_t)(b * ww_)] : nullptr, *zb = b >= 0 ? &zc_[(size_t)(b * ww_)] : nullptr;
    for (int64_t t = 0; t < ww_; ++t) {
        uint64_t &f = fb_[(size_t)t];
        switch (code) {
        case PS_OP_H: {  // :89-93
            const uint64_t x = xa[t], z = za[t];
            f ^= x & z;
            xa[t] = z;
            za[t] = x;
            break;
        }
        case PS_OP_S:  // :164-169
            f ^= xa[t] & za[t];
            za[t] ^= xa[t];
            break;
        case PS_OP_X: f ^= za[t]; break;          // :303-307
        case PS_OP_Y: f ^= za[t] ^ xa[t]; break;  // :323-327
        case PS_OP_Z: f ^= xa[t]; break;          // :372-376
        case PS_OP_CX: {  // :247-253, a = control
            f ^= xa[t] & zb[t] & ~(xb[t] ^ za[t]);
            xb[t] ^= xa[t];
            za[t] ^= zb[t];
            break;
        }
        case PS_OP_CZ: {  // :29-35
            f ^= xa[t] & xb[t] & (zb[t] ^ za[t]);
            zb[t] ^= xa[t];
            za[t] ^= xb[t];
            break;
        }
        default: break;
        }
    }
}

void FrameBuilder::begin_segment(int32_t seg, uint32_t nslots, size_t nops) {
    seg_ = seg;
    seg_col_ = nops >= 64;
    slot_rows_.assign(nslots, {});
}

// Rows whose sign a Pauli on a (b) flips: X flips rows with z set, Z rows
// with x set (the conditional X = H S S H and Z = S S of the channel).
void FrameBuilder::channel(int64_t a, int64_t b, uint32_t slot) {
    std::vector<uint32_t> &rows = slot_rows_[slot];
    rows.clear();
    if (!seg_col_) {
        to_row();
        for (int64_t i = 0; i < W_; ++i) {
            uint32_t sel = (uint32_t)bit(z_, i, a) | (uint32_t)bit(x_, i, a) << 1;
            if (b >= 0) sel |= (uint32_t)bit(z_, i, b) << 2 | (uint32_t)bit(x_, i, b) << 3;
            if (sel) rows.push_back((uint32_t)i | sel << 28);
        }
        return;
    }
    to_col();
    const uint64_t *xa = &xc_[(size_t)(a * ww_)], *za = &zc_[(size_t)(a * ww_)];
    const uint64_t *xb = b >= 0 ? &xc_[(size_t)(b * ww_)] : nullptr, *zb = b >= 0 ? &zc_[(size_t)(b * ww_)] : nullptr;
    for (int64_t t = 0; t < ww_; ++t) {
        uint64_t m = za[t] | xa[t];
        if (b >= 0) m |= zb[t] | xb[t];
        for (; m; m &= m - 1) {
            const int u = __builtin_ctzll(m);
            uint32_t sel = (uint32_t)((za[t] >> u) & 1ull) | (uint32_t)((xa[t] >> u) & 1ull) << 1;
            if (b >= 0) sel |= (uint32_t)((zb[t] >> u) & 1ull) << 2 | (uint32_t)((xb[t] >> u) & 1ull) << 3;
            rows.push_back((uint32_t)(64 * t + u) | sel << 28);
        }
    }
}

void FrameBuilder::end_segment() {
    flush_window();
    if (slot_rows_.empty()) {  // no channels: nothing sampled, nothing to apply
        seg_ = -1;
        return;
    }
    const uint32_t base = (uint32_t)prog.slot_off.size();
    int32_t chunks = 0;
    for (const auto &rows : slot_rows_) {
        prog.slot_off.push_back((uint32_t)prog.tab.size());
        prog.tab.insert(prog.tab.end(), rows.begin(), rows.end());
        chunks += (int32_t)((rows.size() + kFrameChunk - 1) / kFrameChunk);
    }
    prog.entry_cap = std::max(prog.entry_cap, chunks);
    prog.slot_off.push_back((uint32_t)prog.tab.size());
    // A new launch: its sampling precedes it, then this segment's noise.
    if (prog.launches.back().op0 == prog.launches.back().op1) prog.launches.pop_back();
    prog.launches.push_back(
        {seg_, (uint32_t)prog.ops.size(), (uint32_t)prog.ops.size(), 0, 0, (uint32_t)prog.rand_meas.size(), 0});
    FrameOp op{};
    op.kind = F_NOISE;
    op.arg = (int32_t)base;
    push_op(op);
    slot_rows_.clear();
    seg_ = -1;
}

// Bit 1 of the summed phase of row i times row k (RowProductSign,
// MeasurementFunctors.hpp:97-129, the reference's (sum >> 1) & 1).
int FrameBuilder::phase_bit(int64_t i, int64_t k) const {
    long sum = 0;
    for (int64_t t = 0; t < nw_; ++t) {
        const uint64_t x1 = x_[(size_t)(i * nw_ + t)], z1 = z_[(size_t)(i * nw_ + t)];
        const uint64_t x2 = x_[(size_t)(k * nw_ + t)], z2 = z_[(size_t)(k * nw_ + t)];
        const uint64_t plus = (x1 & ~z1 & x2 & z2) | (x1 & z1 & ~x2 & z2) | (~x1 & z1 & x2 & ~z2);
        const uint64_t minus = (x1 & z1 & x2 & ~z2) | (x1 & ~z1 & ~x2 & z2) | (~x1 & z1 & x2 & z2);
        sum += (long)__builtin_popcountll(plus) - (long)__builtin_popcountll(minus);
    }
    return (int)((((sum % 4) + 4) % 4) >> 1);
}

void FrameBuilder::row_xor(int64_t dst, int64_t src) {
    for (int64_t t = 0; t < nw_; ++t) {
        x_[(size_t)(dst * nw_ + t)] ^= x_[(size_t)(src * nw_ + t)];
        z_[(size_t)(dst * nw_ + t)] ^= z_[(size_t)(src * nw_ + t)];
    }
}

// MeasureQubit (CliffordState.hpp:587-623): the lowest stabilizer row p+n
// with x(p+n,q) = 1 takes the random branch, else the deterministic one; a
// reset then flips the rows with z(., q) = 1 where the outcome is 1.
void FrameBuilder::measure(int64_t q, int32_t meas_index, bool reset) {
    to_row();
    const int64_t s = 2 * n_;
    // Column q of rows [0, 2n) from the column-major copy while it is exact
    // (from the last transpose on, only the scratch row has changed).
    const uint64_t *xq = colok_ ? &xc_[(size_t)(q * ww_)] : nullptr;
    const uint64_t *zq = colok_ ? &zc_[(size_t)(q * ww_)] : nullptr;
    int64_t p = 0;
    if (xq)
        p = first_set(xq, n_, 2 * n_) - n_;
    else
        while (p < n_ && !bit(x_, p + n_, q)) ++p;
    if (p < n_) {  // MeasureRandom (:225-265), in program order after the open window
        flush_window();
        std::vector<int64_t> mult;  // rows i < 2n, i != p, p+n, with x(i,q) = 1: rows i themselves are not changed before their turn
        if (xq) {
            each_set(xq, 0, 2 * n_, [&](int64_t i) {
                if (i != p && i != p + n_) mult.push_back(i);
            });
        } else {
            for (int64_t i = 0; i < 2 * n_; ++i)
                if (i != p && i != p + n_ && bit(x_, i, q)) mult.push_back(i);
        }
        colok_ = false;
        FrameOp op{};
        op.kind = F_MEAS_RAND | prog.launches.back().nrand << 8;
        op.arg = meas_index;
        prog.rand_meas.push_back(meas_index);
        prog.launches.back().nrand++;
        op.off = (uint32_t)prog.tab.size();
        prog.tab.push_back((uint32_t)p);
        for (int64_t t = 0; t < nw_; ++t) {  // row p := row p+n; row p+n := Z_q
            x_[(size_t)(p * nw_ + t)] = x_[(size_t)((p + n_) * nw_ + t)];
            z_[(size_t)(p * nw_ + t)] = z_[(size_t)((p + n_) * nw_ + t)];
            x_[(size_t)((p + n_) * nw_ + t)] = 0ull;
            z_[(size_t)((p + n_) * nw_ + t)] = 0ull;
        }
        flip(z_, p + n_, q);
        fset(p, fget(p + n_));
        fset(p + n_, false);
        for (int64_t i : mult) {
            const uint32_t c = (uint32_t)(phase_bit(i, p) ^ (int)fget(p));
            prog.tab.push_back((uint32_t)i | c << 31);
            row_xor(i, p);
        }
        op.len = (uint32_t)prog.tab.size() - op.off;
        push_op(op);
        if (reset) {
            FrameOp ro{};
            ro.kind = F_RESET_X;
            ro.off = (uint32_t)prog.tab.size();
            for (int64_t i = 0; i < W_; ++i)
                if (bit(z_, i, q)) prog.tab.push_back((uint32_t)i);
            ro.len = (uint32_t)prog.tab.size() - ro.off;
            push_op(ro);
        }
        return;
    }
    // MeasureDetermined (:189-201): scratch row := product of the selected stabilizers
    DetRecord r;
    r.meas = meas_index;
    for (int64_t t = 0; t < nw_; ++t) {
        x_[(size_t)(s * nw_ + t)] = 0ull;
        z_[(size_t)(s * nw_ + t)] = 0ull;
    }
    uint32_t c = 0;
    auto take = [&](int64_t i) {
        c ^= (uint32_t)(phase_bit(s, i + n_) ^ (int)fget(i + n_));
        r.rd.push_back((uint32_t)(i + n_));
        row_xor(s, i + n_);
    };
    if (xq) {
        each_set(xq, 0, n_, take);
    } else {
        for (int64_t i = 0; i < n_; ++i)
            if (bit(x_, i, q)) take(i);
    }
    r.c = c;
    fset(s, false);
    if (reset) {
        if (zq) {
            each_set(zq, 0, 2 * n_, [&](int64_t i) { r.rs.push_back((uint32_t)i); });
            if (bit(z_, s, q)) r.rs.push_back((uint32_t)s);
        } else {
            for (int64_t i = 0; i < W_; ++i)
                if (bit(z_, i, q)) r.rs.push_back((uint32_t)i);
        }
    }
    if (r.rd.size() > kWinRows || r.rs.size() > kWinRows) {  // too long for a window record: alone
        flush_window();
        FrameOp op{};
        op.kind = F_MEAS_DET | r.c << 8;
        op.arg = meas_index;
        op.off = (uint32_t)prog.tab.size();
        prog.tab.insert(prog.tab.end(), r.rd.begin(), r.rd.end());
        op.len = (uint32_t)r.rd.size();
        push_op(op);
        if (reset) {
            FrameOp ro{};
            ro.kind = F_RESET_X;
            ro.off = (uint32_t)prog.tab.size();
            prog.tab.insert(prog.tab.end(), r.rs.begin(), r.rs.end());
            ro.len = (uint32_t)r.rs.size();
            push_op(ro);
        }
        return;
    }
    bool hazard = window_.size() == 32;
    for (uint32_t row : r.rd) hazard |= flipped_[row] == stamp_;  // reads a row a reset of the window flips
    for (uint32_t row : r.rs)
        if (row != (uint32_t)s) hazard |= flipped_[row] == stamp_;  // flips a row a reset of the window flips
    if (hazard) flush_window();
    for (uint32_t row : r.rs)
        if (row != (uint32_t)s) flipped_[row] = stamp_;
    window_.push_back(std::move(r));
}

void FrameBuilder::finish() {
    to_row();
    flush_window();
    FrameOp op{};
    op.kind = F_FLIP;
    op.off = (uint32_t)prog.tab.size();
    for (int64_t i = 0; i < W_; ++i)
        if (fget(i)) prog.tab.push_back((uint32_t)i);
    op.len = (uint32_t)prog.tab.size() - op.off;
    push_op(op);
    for (FrameProgram::Launch &L : prog.launches) {  // tab range of the measurement ops
        L.tab0 = L.tab1 = 0;
        bool any = false;
        for (uint32_t i = L.op0; i < L.op1; ++i) {
            if ((prog.ops[i].kind & 0xFFu) == F_NOISE) continue;
            if (!any) L.tab0 = prog.ops[i].off;
            L.tab1 = op_tab_end_[i];
            any = true;
        }
    }
    prog.xz.assign((size_t)(W_ * 2 * nw_), 0ull);
    for (int64_t i = 0; i < W_; ++i)
        for (int64_t t = 0; t < nw_; ++t) {
            prog.xz[(size_t)((i * 2 + 0) * nw_ + t)] = x_[(size_t)(i * nw_ + t)];
            prog.xz[(size_t)((i * 2 + 1) * nw_ + t)] = z_[(size_t)(i * nw_ + t)];
        }
}

namespace {

// An affine form over GF(2): sorted input indices (shared-memory sign
// indices, see F_LINEAR) and a constant.
struct Form {
    std::vector<uint32_t> t;
    bool c = false;
};

void xor_into(Form &a, const Form &b) {
    a.c ^= b.c;
    if (b.t.empty()) return;
    std::vector<uint32_t> out;
    out.reserve(a.t.size() + b.t.size());
    std::set_symmetric_difference(a.t.begin(), a.t.end(), b.t.begin(), b.t.end(), std::back_inserter(out));
    a.t.swap(out);
}

// Largest F_LINEAR record (words of tab; a launch stages its measurement
// rows in shared memory) and the terms a run may cost per op it replaces:
// one op on one warp is a chain of a few dependent shared-memory steps,
// while the CTA's 128 threads evaluate about that many terms in the same
// time.
constexpr size_t kLinWordsMax = 16384;
constexpr size_t kLinTermsPerOp = 512;

// The sign program's measurement ops executed on forms instead of signs,
// exactly as frame_kernel runs them: the signs at the start of a run are
// the inputs (row i = {i}), a random outcome r is {kLinRand0(W) + r}.  Every
// op can be taken back, so a run is cut where its map outgrows the budget.
class PhaseMap {
  public:
    PhaseMap(int64_t n, const std::vector<uint32_t> &tab)
        : n_((uint32_t)n), W_((uint32_t)(2 * n + 1)), tab_(tab), stamp_(W_, 0), logged_(W_, 0), form_(W_) {}

    void reset() {
        ++cur_;
        touched_.clear();
        recs_.clear();
        has_last_ = false;
        last_ = Form{};
        rec_terms_ = row_terms_ = 0;
        nops_ = 0;
    }
    size_t nops() const { return nops_; }

    // false (and nothing applied) for a reset X whose outcome the run does not hold
    bool apply(const FrameOp &o) {
        const uint32_t kind = o.kind & 0xFFu;
        if (kind == F_RESET_X && !has_last_) return false;
        sv_ = {recs_.size(), touched_.size(), rec_terms_, row_terms_, has_last_};
        sv_last_ = last_;
        ++op_;
        log_.clear();
        const uint32_t s = 2 * n_;
        if (kind == F_WINDOW) {
            std::vector<Form> acc(o.len);
            for (uint32_t j = 0; j < o.len; ++j) {
                const uint32_t *rc = &tab_[o.off + kWinRec * j];
                acc[j].c = rc[1] & 1u;
                for (uint32_t t = 0; t < kWinRows; ++t) xor_into(acc[j], get(rc[2 + t]));
                record(rc[0] | kLinDet, acc[j]);
            }
            mut(s) = acc[o.len - 1];
            for (uint32_t j = 0; j < o.len; ++j)
                for (uint32_t t = 0; t < kWinRows; ++t) {
                    const uint32_t r = tab_[o.off + kWinRec * j + 2 + kWinRows + t];
                    if (r < W_) xor_into(mut(r), acc[j]);
                }
            set_last(acc[o.len - 1]);
        } else if (kind == F_MEAS_DET) {
            Form a;
            a.c = (o.kind >> 8) != 0u;
            for (uint32_t t = o.off; t < o.off + o.len; ++t) xor_into(a, get(tab_[t]));
            record((uint32_t)o.arg | kLinDet, a);
            mut(s) = a;
            set_last(a);
        } else if (kind == F_MEAS_RAND) {
            const uint32_t p = tab_[o.off];
            const Form rpv = get(p + n_);
            Form out;
            out.t.push_back(kLinRand0(W_) + (o.kind >> 8));
            mut(p) = rpv;
            mut(p + n_) = out;
            record((uint32_t)o.arg, out);
            for (uint32_t t = o.off + 1; t < o.off + o.len; ++t) {
                Form &f = mut(tab_[t] & 0x7FFFFFFFu);
                xor_into(f, rpv);
                f.c ^= (tab_[t] >> 31) != 0u;
            }
            set_last(out);
        } else {  // F_RESET_X, F_FLIP
            for (uint32_t t = o.off; t < o.off + o.len; ++t) {
                const uint32_t r = tab_[t];
                if (r >= W_) continue;
                if (kind == F_RESET_X)
                    xor_into(mut(r), last_);
                else
                    mut(r).c ^= true;
            }
        }
        for (const Log &l : log_) row_terms_ += form_[l.row].t.size() - (l.was ? l.old.t.size() : 0);
        ++nops_;
        return true;
    }

    void undo() {
        for (size_t i = log_.size(); i-- > 0;) {
            const Log &l = log_[i];
            form_[l.row] = l.old;
            if (!l.was) stamp_[l.row] = 0;
        }
        log_.clear();
        recs_.resize(sv_.nrec);
        touched_.resize(sv_.ntouched);
        rec_terms_ = sv_.rec_terms;
        row_terms_ = sv_.row_terms;
        has_last_ = sv_.has_last;
        last_ = sv_last_;
        --nops_;
    }

    bool over(uint32_t max_rows, size_t ops) const {
        const size_t terms = rec_terms_ + row_terms_ + last_.t.size();
        const size_t nout = recs_.size() + touched_.size() + 1;
        return touched_.size() + 1 > max_rows || 5 + 2 * nout + terms > kLinWordsMax ||
               terms > kLinTermsPerOp * (ops + 1);
    }

    // The run as one F_LINEAR op (appended to tab); scratch: its new-row words.
    FrameOp emit(std::vector<uint32_t> &tab, uint32_t *scratch) const {
        std::vector<uint32_t> rows;
        for (uint32_t r : touched_) {
            const Form &f = form_[r];
            if (!(f.c == false && f.t.size() == 1 && f.t[0] == r)) rows.push_back(r);
        }
        std::sort(rows.begin(), rows.end());
        const uint32_t nrec = (uint32_t)recs_.size(), nrow = (uint32_t)rows.size(), nlast = has_last_ ? 1u : 0u;
        const uint32_t nout = nrec + nrow + nlast;
        FrameOp op{};
        op.kind = F_LINEAR;
        op.off = (uint32_t)tab.size();
        tab.push_back(nrec);
        tab.push_back(nrow);
        tab.push_back(nlast);
        tab.push_back(0u);
        for (const Rec &r : recs_) tab.push_back(r.dst | (r.f.c ? kLinConst : 0u));
        for (uint32_t r : rows) tab.push_back(r | (form_[r].c ? kLinConst : 0u));
        if (nlast) tab.push_back(last_.c ? kLinConst : 0u);
        uint32_t b = 0;
        tab.push_back(b);
        for (const Rec &r : recs_) tab.push_back(b += (uint32_t)r.f.t.size());
        for (uint32_t r : rows) tab.push_back(b += (uint32_t)form_[r].t.size());
        if (nlast) tab.push_back(b += (uint32_t)last_.t.size());
        for (const Rec &r : recs_) tab.insert(tab.end(), r.f.t.begin(), r.f.t.end());
        for (uint32_t r : rows) tab.insert(tab.end(), form_[r].t.begin(), form_[r].t.end());
        if (nlast) tab.insert(tab.end(), last_.t.begin(), last_.t.end());
        op.len = (uint32_t)tab.size() - op.off;
        *scratch = nrow + nlast;
        (void)nout;
        return op;
    }

  private:
    struct Rec {
        uint32_t dst;
        Form f;
    };
    struct Log {
        uint32_t row;
        bool was;  // touched before this op
        Form old;
    };
    struct Saved {
        size_t nrec, ntouched, rec_terms, row_terms;
        bool has_last;
    };
    uint32_t n_, W_;
    const std::vector<uint32_t> &tab_;
    std::vector<uint32_t> stamp_, logged_;  // row -> run that touched it, op that logged it
    std::vector<Form> form_;
    std::vector<uint32_t> touched_;
    std::vector<Rec> recs_;
    std::vector<Log> log_;
    Form last_, sv_last_;
    bool has_last_ = false;
    size_t rec_terms_ = 0, row_terms_ = 0, nops_ = 0;
    uint32_t cur_ = 0, op_ = 0;
    Saved sv_{};

    Form get(uint32_t r) const {  // the zero row and the sinks read as 0
        if (r >= W_) return Form{};
        if (stamp_[r] != cur_) return Form{{r}, false};
        return form_[r];
    }
    Form &mut(uint32_t r) {
        const bool was = stamp_[r] == cur_;
        if (logged_[r] != op_) {
            logged_[r] = op_;
            log_.push_back({r, was, was ? form_[r] : Form{}});
        }
        if (!was) {
            stamp_[r] = cur_;
            form_[r] = Form{{r}, false};
            touched_.push_back(r);
        }
        return form_[r];
    }
    void record(uint32_t dst, const Form &f) {
        recs_.push_back({dst, f});
        rec_terms_ += f.t.size();
    }
    void set_last(const Form &f) {
        last_ = f;
        has_last_ = true;
    }
};

}  // namespace

void FrameBuilder::linearize(uint32_t max_rows) {
    if (max_rows < 2) return;
    const std::vector<FrameOp> old = prog.ops;
    std::vector<uint32_t> &tab = prog.tab;
    std::vector<FrameOp> ops;
    PhaseMap pm(n_, tab);
    for (FrameProgram::Launch &L : prog.launches) {
        // The launch's measurement ops, linear or kept, get a fresh
        // contiguous tab range (the staged one).
        const uint32_t new0 = (uint32_t)ops.size(), t0 = (uint32_t)tab.size();
        std::vector<uint32_t> run;  // old indices of the ops in pm
        L.scratch = 0;
        auto keep = [&](uint32_t i) {
            FrameOp o = old[i];
            if ((o.kind & 0xFFu) != F_NOISE) {
                const uint32_t a = o.off, b = op_tab_end_[i];
                o.off = (uint32_t)tab.size();
                for (uint32_t t = a; t < b; ++t) {
                    const uint32_t v = tab[t];
                    tab.push_back(v);
                }
            }
            ops.push_back(o);
        };
        auto flush = [&]() {
            if (pm.nops() >= 2) {
                uint32_t s = 0;
                ops.push_back(pm.emit(tab, &s));
                L.scratch = std::max(L.scratch, s);
            } else {
                for (uint32_t i : run) keep(i);
            }
            run.clear();
            pm.reset();
        };
        pm.reset();
        for (uint32_t i = L.op0; i < L.op1; ++i) {
            if ((old[i].kind & 0xFFu) == F_NOISE) {
                flush();
                keep(i);
                continue;
            }
            bool applied = pm.apply(old[i]);
            if (applied && pm.over(max_rows, run.size() + 1)) {
                pm.undo();
                flush();
                applied = pm.apply(old[i]);
                if (applied && pm.over(max_rows, 1)) {
                    pm.undo();
                    applied = false;
                }
            }
            if (applied) {
                run.push_back(i);
            } else {  // on its own, between the runs before and after it
                flush();
                keep(i);
            }
        }
        flush();
        L.op0 = new0;
        L.op1 = (uint32_t)ops.size();
        L.tab0 = t0;
        L.tab1 = (uint32_t)tab.size();
    }
    prog.ops.swap(ops);
    op_tab_end_.clear();
}

}  // namespace ps
