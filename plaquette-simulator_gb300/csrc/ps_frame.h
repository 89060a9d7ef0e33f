// ps_frame.h -- shared-x/z runs of compiled circuits.
//
// Clifford gates, Pauli gates, Pauli channels and Z measurements (with their
// resets) never make the x / z bits of one shot's tableau differ from
// another's: a Pauli only flips signs (the conditional X / Z of a channel or
// a reset is H S S H / S S with the shot's flag, which leaves x / z as they
// were, GateFunctors.hpp:142-148, :220-228), the random branch of a
// measurement picks its pivot from x / z alone (MeasurementFunctors.hpp:
// 297-301), and every sign update is r_i ^ r_k ^ (a bit of a phase sum over
// x / z) (:97-129).  Only the per-shot conditional H / S gates break this.
// So from |0...0> the x / z bits of every tableau row are one host-side
// simulation, and what each shot-word has of its own are the signs R[row]:
// a run becomes a program of XORs between sign rows whose row lists and
// constants the host computes while simulating x / z:
//   noise      R[i] ^= fx / fz of a sampled channel outcome, rows i whose x / z
//              anticommute with that Pauli at the channel's position;
//   det. meas. outcome = c ^ XOR of R[i+n] over the destabilizers i with
//              x(i,q) = 1 (MeasureDetermined, :189-201), into record and
//              scratch row;
//   rand. meas R[p] := R[p+n]; R[p+n] := drawn outcome; R[i] ^= R[p] ^ c_i
//              for the rows the reference multiplies (MeasureRandom,
//              :225-265);
//   reset X    R[i] ^= outcome for rows with z(i,q) = 1;
// and the sign flips of gates and Pauli gates are constants folded into
// those c's (the device keeps R ^ F for a host-known row mask F, applied at
// the end).  The final x / z bits are broadcast to every shot, so the state
// ends exactly as the per-shot plan leaves it.
#pragma once
#include <stdint.h>

#include <vector>

namespace ps {

enum FrameKind : uint32_t {
    F_NOISE = 0,      // segment noise, the range's first op: arg = slot_off index of its first slot
    F_MEAS_DET = 1,   // arg = MeasOp; tab[off..off+len) rows; kind bit 8 = constant (more rows than a window record holds)
    F_MEAS_RAND = 2,  // arg = MeasOp; tab[off] = p, then rows | c << 31; kind >> 8 = its index in the launch's random list
    F_RESET_X = 3,    // R[row] ^= outcome of the last measurement, rows tab[off..off+len)
    F_FLIP = 4,       // R[row] ^= ~0, rows tab[off..off+len)
    F_WINDOW = 5,     // len deterministic measurements, one per lane (below)
    F_LINEAR = 6,     // a run of the ops above as one linear map over the signs (below); arg unused
};

// A window of deterministic measurements (each with its reset X) that run
// at once, one per lane: every lane reads its rows first, the last one
// writes the scratch row, then the resets XOR their outcomes in.  The
// builder closes a window before a measurement that reads a row an earlier
// reset of the window flips, or whose reset flips a row an earlier reset
// flips (so the XORs need no atomics; a reset that flips a row an earlier
// measurement read is fine: reads come first), and drops the scratch row
// from every reset but the last one's (the last measurement overwrites it).
// Record j sits at tab[off + kWinRec * j]: [MeasOp index][c | nread << 1 |
// nreset << 4][kWinRows read rows][kWinRows reset rows], unused read rows
// pointing at the zero row W and unused reset row t at the sink row W+1+t
// (a lane's reset rows are then distinct).
constexpr uint32_t kWinRows = 4;
constexpr uint32_t kWinRec = 2 + 2 * kWinRows;

// Between two channel ops every op above is affine over GF(2) in the signs
// it starts from and the launch's random outcomes (drawn up front), so a run
// of them is, for every record it writes, every row it changes and the
// latest outcome (read by a later reset X), a constant XOR a set of inputs.
// An F_LINEAR op holds those sets; all threads of the CTA evaluate them at
// once, then write the changed rows, instead of one warp stepping through the
// run.  tab[off..off+len): [nrec][nrow][nlast][0], dst[nout], beg[nout + 1],
// terms, nout = nrec + nrow + nlast (records, changed rows, the latest
// outcome), output j = const XOR sR[terms[beg[j] .. beg[j+1])], a term being
// a shared-memory sign index (rows < W, random outcome r at kLinRand0(W) + r).
// dst: record MeasOp index | kLinConst | kLinDet (determined), or row |
// kLinConst.
constexpr uint32_t kLinIndex = 0x3FFFFFFFu;
constexpr uint32_t kLinConst = 1u << 30;
constexpr uint32_t kLinDet = 1u << 31;
inline uint32_t kLinRand0(int64_t W) { return (uint32_t)W + 1 + kWinRows; }

struct FrameOp {
    uint32_t kind;  // FrameKind | constant bit << 8
    int32_t arg;    // MeasOp index, or for F_NOISE the offset of the segment's slot table
    uint32_t off;   // into tab
    uint32_t len;
};

// Noise table entry: row | sel << 28, sel bit 0 fx(a), 1 fz(a), 2 fx(b), 3 fz(b).
constexpr uint32_t kFrameRowMask = 0x0FFFFFFFu;
// A sampled outcome is applied in chunks of at most this many rows.
constexpr uint32_t kFrameChunk = 16;

struct FrameProgram {
    std::vector<FrameOp> ops;
    std::vector<uint32_t> tab;
    std::vector<uint32_t> slot_off;  // per segment: nslots + 1 offsets into tab
    int32_t entry_cap = 0;           // largest sum over a segment's slots of its row chunks
    std::vector<uint64_t> xz;        // final x / z bits: [W][2][nw64]
    int64_t nw64 = 0;
    // op ranges launched together: the ops of one segment's noise and the
    // measurement phase after it (seg = -1: no sampling before the range)
    struct Launch {
        int32_t seg;
        uint32_t op0, op1;
        uint32_t tab0, tab1;  // tab range of the launch's measurement ops (staged in shared memory)
        uint32_t rand0, nrand;  // the launch's random measurements: rand_meas[rand0, rand0 + nrand)
        uint32_t scratch = 0;   // shared-memory words its F_LINEAR ops stage new rows in (nrow + nlast)
    };
    // MeasOp indices of the random measurements, launch by launch: their
    // outcomes depend on no sign, so a launch draws them all up front.
    std::vector<int32_t> rand_meas;
    std::vector<Launch> launches;
};

// Host-side simulation of the shared x / z bits and emission of the sign
// program.  Calls follow the circuit's program order.
class FrameBuilder {
  public:
    explicit FrameBuilder(int64_t n);
    void gate(int32_t code, int64_t a, int64_t b);  // H, S, X, Y, Z, CX, CZ
    // Pauli channel on a (and b >= 0): slot `slot` of the current segment.
    void channel(int64_t a, int64_t b, uint32_t slot);
    // nops: the segment's op count (a long one is simulated column-major).
    void begin_segment(int32_t seg, uint32_t nslots, size_t nops);
    void end_segment();
    void measure(int64_t q, int32_t meas_index, bool reset);
    void finish();
    // After finish(): every run of two or more measurement-phase ops becomes
    // F_LINEAR ops whose new rows take at most max_rows words of shared
    // memory (0: none), where that costs the device fewer steps.
    void linearize(uint32_t max_rows);
    FrameProgram prog;

    struct DetRecord {
        int32_t meas;
        uint32_t c;
        std::vector<uint32_t> rd, rs;
    };

  private:
    // x / z are kept column-major ([n][ww], word-parallel gates over rows)
    // while a long segment is simulated and row-major ([W][nw], row
    // products) otherwise; switching transposes by the set bits.
    int64_t n_, W_, nw_, ww_;
    std::vector<uint64_t> x_, z_;    // row-major [W][nw]
    std::vector<uint64_t> xc_, zc_;  // column-major [n][ww]
    bool col_ = false;
    bool colok_ = false;    // row-major mode: the column-major copy is exact but for the scratch row
    bool seg_col_ = false;  // the current segment runs column-major
    std::vector<uint64_t> fb_;       // pending constant flips, a bit per row
    bool fget(int64_t i) const { return (fb_[(size_t)(i >> 6)] >> (i & 63)) & 1ull; }
    void fset(int64_t i, bool v) {
        const uint64_t m = 1ull << (i & 63);
        fb_[(size_t)(i >> 6)] = v ? (fb_[(size_t)(i >> 6)] | m) : (fb_[(size_t)(i >> 6)] & ~m);
    }
    void to_col();
    void to_row();
    int32_t seg_ = -1;
    std::vector<std::vector<uint32_t>> slot_rows_;
    std::vector<DetRecord> window_;
    std::vector<uint32_t> flipped_;  // row -> window stamp of a reset flip in the open window
    uint32_t stamp_ = 1;
    std::vector<uint32_t> op_tab_end_;  // tab extent end of every op
    void flush_window();
    void push_op(const FrameOp &op);
    bool bit(const std::vector<uint64_t> &m, int64_t row, int64_t q) const {
        return (m[(size_t)(row * nw_ + (q >> 6))] >> (q & 63)) & 1ull;
    }
    void flip(std::vector<uint64_t> &m, int64_t row, int64_t q) { m[(size_t)(row * nw_ + (q >> 6))] ^= 1ull << (q & 63); }
    int phase_bit(int64_t i, int64_t k) const;  // bit 1 of the summed phase of row i times row k
    void row_xor(int64_t dst, int64_t src);
    void open_range();
};

}  // namespace ps
