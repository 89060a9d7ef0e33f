/*
 * ps_oracle.c -- CPU oracle (test infrastructure only; see ps_oracle.h).
 *
 * Every function restates the reference's algorithm in its own storage
 * layout (int32 per bit, [shot][row][qubit], W = 2n+1 rows) and cites the
 * reference file:line it follows.  Parallelism is OpenMP over shots, which is
 * what the reference's Kokkos OpenMP backend does for its MDRange/Range
 * policies (CliffordState.hpp:381-386, :590).
 */
#include "ps_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ RNG */
/* Philox4x32-10, written from the published description: each round maps
 * (c0,c1,c2,c3) to (hi(M1*c2)^c1^k0, lo(M1*c2), hi(M0*c0)^c3^k1, lo(M0*c0))
 * and the key is bumped by the Weyl constants between rounds. */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

enum { TAG_MEASURE = 1, TAG_NOISE = 2, TAG_NOISE_FIRST = 3 };

/* One 32-bit draw for (seed, event, global shot, tag), the draw of a
 * random measurement's shot.  Shot g lives in 64-shot word g>>6; the word's
 * 64 draws come from 16 Philox blocks with counter (sub, word, event, tag),
 * sub = (g&63)>>2, lane = g&3.  (Pauli channels draw per word instead:
 * ora_channel_paulis.) */
uint32_t ora_draw_u32(int64_t seed, uint64_t event, int64_t gshot, uint32_t tag) {
    uint32_t key[2] = {(uint32_t)((uint64_t)seed & 0xffffffffu), (uint32_t)((uint64_t)seed >> 32)};
    uint64_t word = (uint64_t)gshot >> 6;
    uint32_t ctr[4] = {(uint32_t)(((uint64_t)gshot & 63u) >> 2), (uint32_t)word, (uint32_t)event, tag};
    uint32_t out[4];
    ora_philox4x32_10(ctr, key, out);
    return out[gshot & 3];
}

/* Uniform float in [0,1) with 24 random bits; exact in binary32. */
static float u32_to_unit_float(uint32_t u) { return (float)(u >> 8) * (1.0f / 16777216.0f); }

uint64_t ora_threshold(double cumulative) {
    if (!(cumulative > 0.0)) return 0;
    if (cumulative >= 1.0) return (uint64_t)1 << 32;
    double t = floor(cumulative * 4294967296.0);
    return (uint64_t)t;
}

/* --------------------------------------------------------------- state */
typedef struct {
    int64_t qubit;
    int32_t *res;
    int32_t *det;
} ora_record;

struct ora_state {
    int64_t n, batch, W, seed, shot_base;
    uint64_t events;
    int32_t *x, *z, *r;
    ora_record *recs;
    int64_t nrecs, caprecs;
};

static int g_threads = 0;
void ora_set_threads(int nthreads) { g_threads = nthreads; }
#ifdef _OPENMP
#define OMP_THREADS() (g_threads > 0 ? g_threads : omp_get_max_threads())
#else
#define OMP_THREADS() 1
#endif

#define XI(s, b, i, j) ((s)->x[((b) * (s)->W + (i)) * (s)->n + (j)])
#define ZI(s, b, i, j) ((s)->z[((b) * (s)->W + (i)) * (s)->n + (j)])
#define RI(s, b, i) ((s)->r[(b) * (s)->W + (i)])

/* InitTableauToZeroStateFunctor (MiscFunctors.hpp:8-28) over the ctor's
 * policy {B, W, n} (CliffordState.hpp:122-127): x(i,j)=[i==j],
 * z(i,j)=[i-n==j], r(i)=[i==2n]. */
static void init_zero(ora_state *s) {
    const int64_t n = s->n, W = s->W;
#pragma omp parallel for num_threads(OMP_THREADS()) schedule(static)
    for (int64_t b = 0; b < s->batch; ++b) {
        for (int64_t i = 0; i < W; ++i) {
            for (int64_t j = 0; j < n; ++j) {
                XI(s, b, i, j) = (i == j);
                ZI(s, b, i, j) = (i - n == j);
            }
            RI(s, b, i) = (i == 2 * n);
        }
    }
}

ora_state *ora_create(int64_t n, int64_t batch, int64_t seed, int init_zero_state, int64_t shot_base) {
    ora_state *s = (ora_state *)calloc(1, sizeof(ora_state));
    s->n = n;
    s->batch = batch;
    s->W = 2 * n + 1;
    /* CliffordState.hpp:130-138: negative seed falls back to 213434232223. */
    s->seed = seed >= 0 ? seed : 213434232223LL;
    s->shot_base = shot_base;
    size_t cells = (size_t)(batch * s->W * n);
    s->x = (int32_t *)calloc(cells ? cells : 1, sizeof(int32_t));
    s->z = (int32_t *)calloc(cells ? cells : 1, sizeof(int32_t));
    s->r = (int32_t *)calloc((size_t)(batch * s->W) ? (size_t)(batch * s->W) : 1, sizeof(int32_t));
    if (init_zero_state && n > 0 && batch > 0) init_zero(s);
    return s;
}

ora_state *ora_create_from_host(const int32_t *x, const int32_t *z, const int32_t *r, int64_t n,
                                int64_t batch, int64_t seed, int64_t shot_base) {
    ora_state *s = ora_create(n, batch, seed, 0, shot_base);
    ora_host_to_device(s, x, z, r);
    return s;
}

ora_state *ora_clone(const ora_state *o) {
    ora_state *s = ora_create(o->n, o->batch, o->seed, 0, o->shot_base);
    ora_host_to_device(s, o->x, o->z, o->r);
    s->events = o->events;
    return s;
}

void ora_destroy(ora_state *s) {
    if (!s) return;
    for (int64_t k = 0; k < s->nrecs; ++k) {
        free(s->recs[k].res);
        free(s->recs[k].det);
    }
    free(s->recs);
    free(s->x);
    free(s->z);
    free(s->r);
    free(s);
}

int64_t ora_num_qubits(const ora_state *s) { return s->n; }
int64_t ora_batch(const ora_state *s) { return s->batch; }
int64_t ora_seed(const ora_state *s) { return s->seed; }
uint64_t ora_events(const ora_state *s) { return s->events; }
int32_t *ora_x(ora_state *s) { return s->x; }
int32_t *ora_z(ora_state *s) { return s->z; }
int32_t *ora_r(ora_state *s) { return s->r; }

void ora_device_to_host(const ora_state *s, int32_t *x, int32_t *z, int32_t *r) {
    size_t cells = (size_t)(s->batch * s->W * s->n);
    memcpy(x, s->x, cells * sizeof(int32_t));
    memcpy(z, s->z, cells * sizeof(int32_t));
    memcpy(r, s->r, (size_t)(s->batch * s->W) * sizeof(int32_t));
}

void ora_host_to_device(ora_state *s, const int32_t *x, const int32_t *z, const int32_t *r) {
    size_t cells = (size_t)(s->batch * s->W * s->n);
    memcpy(s->x, x, cells * sizeof(int32_t));
    memcpy(s->z, z, cells * sizeof(int32_t));
    memcpy(s->r, r, (size_t)(s->batch * s->W) * sizeof(int32_t));
}

/* ResetCliffordState (CliffordState.hpp:309-316) launches the init functor
 * over {B, W, W}, which writes past each shot's rows.  The oracle implements
 * the intended result instead: the same tableau as a fresh constructor. */
void ora_reset(ora_state *s) {
    if (s->n > 0 && s->batch > 0) init_zero(s);
}

/* CheckSum / CheckSumFunctor (CliffordState.hpp:327-338,
 * MiscFunctors.hpp:30-50): sum of every x, z and r entry over [s0, s1). */
int64_t ora_checksum(const ora_state *s, int64_t s0, int64_t s1) {
    if (s1 < 0) s1 = s->batch;
    int64_t sum = 0;
    for (int64_t b = s0; b < s1; ++b)
        for (int64_t i = 0; i < s->W; ++i) {
            sum += RI(s, b, i);
            for (int64_t j = 0; j < s->n; ++j) sum += XI(s, b, i, j) + ZI(s, b, i, j);
        }
    return sum;
}

/* ---------------------------------------------------------------- gates */
/* Each gate runs over every (shot, row) pair including the scratch row, as
 * the reference's MDRange policy {B, W} does (CliffordState.hpp:381-386). */
#define FOR_ALL_ROWS(s) \
    _Pragma("omp parallel for num_threads(OMP_THREADS()) schedule(static)") \
    for (int64_t b = 0; b < (s)->batch; ++b) \
        for (int64_t i = 0; i < (s)->W; ++i)

/* BatchHadamardGateFunctor (GateFunctors.hpp:89-93). */
void ora_h(ora_state *s, int64_t q) {
    FOR_ALL_ROWS(s) {
        int32_t xv = XI(s, b, i, q), zv = ZI(s, b, i, q);
        RI(s, b, i) ^= xv & zv;
        XI(s, b, i, q) = zv;
        ZI(s, b, i, q) = xv;
    }
}

/* BatchPhaseGateFunctor (GateFunctors.hpp:164-169). */
void ora_s(ora_state *s, int64_t q) {
    FOR_ALL_ROWS(s) {
        int32_t xv = XI(s, b, i, q);
        RI(s, b, i) ^= xv & ZI(s, b, i, q);
        ZI(s, b, i, q) ^= xv;
    }
}

/* BatchPauliXGateFunctor (GateFunctors.hpp:303-307): r ^= z_q. */
void ora_x_gate(ora_state *s, int64_t q) {
    FOR_ALL_ROWS(s) { RI(s, b, i) ^= ZI(s, b, i, q); }
}

/* BatchPauliYGateFunctor (GateFunctors.hpp:323-327): r ^= z_q ^ x_q. */
void ora_y_gate(ora_state *s, int64_t q) {
    FOR_ALL_ROWS(s) { RI(s, b, i) ^= ZI(s, b, i, q) ^ XI(s, b, i, q); }
}

/* BatchPauliZGateFunctor (GateFunctors.hpp:372-376): r ^= x_q. */
void ora_z_gate(ora_state *s, int64_t q) {
    FOR_ALL_ROWS(s) { RI(s, b, i) ^= XI(s, b, i, q); }
}

/* BatchControlNotGateFunctor (GateFunctors.hpp:247-253). */
void ora_cx(ora_state *s, int64_t c, int64_t t) {
    FOR_ALL_ROWS(s) {
        int32_t xc = XI(s, b, i, c), zc = ZI(s, b, i, c), xt = XI(s, b, i, t), zt = ZI(s, b, i, t);
        RI(s, b, i) ^= xc & zt & (xt ^ zc ^ 1);
        XI(s, b, i, t) = xt ^ xc;
        ZI(s, b, i, c) = zc ^ zt;
    }
}

/* BatchControlPhaseGateFunctor (GateFunctors.hpp:29-35). */
void ora_cz(ora_state *s, int64_t c, int64_t t) {
    FOR_ALL_ROWS(s) {
        int32_t xc = XI(s, b, i, c), zc = ZI(s, b, i, c), xt = XI(s, b, i, t), zt = ZI(s, b, i, t);
        RI(s, b, i) ^= xc * xt * (zt ^ zc);
        ZI(s, b, i, t) = zt ^ xc;
        ZI(s, b, i, c) = zc ^ xt;
    }
}

/* BatchHadamardGateWithApplyFlagFunctor (GateFunctors.hpp:142-148). */
void ora_h_flag(ora_state *s, int64_t q, const int32_t *flag) {
    FOR_ALL_ROWS(s) {
        if (flag[b]) {
            int32_t xv = XI(s, b, i, q), zv = ZI(s, b, i, q);
            RI(s, b, i) ^= xv & zv;
            XI(s, b, i, q) = zv;
            ZI(s, b, i, q) = xv;
        }
    }
}

/* BatchPhaseGateWithApplyFlagFunctor (GateFunctors.hpp:220-228). */
void ora_s_flag(ora_state *s, int64_t q, const int32_t *flag) {
    FOR_ALL_ROWS(s) {
        if (flag[b]) {
            int32_t xv = XI(s, b, i, q);
            RI(s, b, i) ^= xv & ZI(s, b, i, q);
            ZI(s, b, i, q) ^= xv;
        }
    }
}

/* ---------------------------------------------------------- measurement */
/* PauliProductPhase (MeasurementFunctors.hpp:10-72): the exponent g of i in
 * P1*P2 for single-qubit Paulis (x1,z1),(x2,z2); table pinned by
 * Test_CliffordState.hpp:160-174. */
int32_t ora_pauli_product_phase(int32_t x1, int32_t z1, int32_t x2, int32_t z2) {
    if (x1 == 1 && z1 == 1) { /* Y */
        if (x2 == 0 && z2 == 0) return 0;
        if (x2 == 1 && z2 == 0) return -1;
        if (x2 == 1 && z2 == 1) return 0;
        return 1;
    }
    if (x1 == 1 && z1 == 0) { /* X */
        if (x2 == 0 && z2 == 0) return 0;
        if (x2 == 1 && z2 == 0) return 0;
        if (x2 == 1 && z2 == 1) return 1;
        return -1;
    }
    if (z1 == 1 && x1 == 0) { /* Z */
        if (x2 == 0 && z2 == 0) return 0;
        if (x2 == 1 && z2 == 0) return 1;
        if (x2 == 1 && z2 == 1) return -1;
        return 0;
    }
    return 0;
}

/* RowProductSign (MeasurementFunctors.hpp:97-129): r_i ^ r_k ^ bit 1 of the
 * summed phase.  The reference takes (sum >> 1) & 1 of an int; for a
 * two's-complement int that is bit 1 of (sum mod 4), written here without
 * relying on the shift of a negative value. */
static int32_t row_product_sign(const ora_state *s, int64_t b, int64_t i, int64_t k) {
    int64_t sum = 0;
    for (int64_t j = 0; j < s->n; ++j)
        sum += ora_pauli_product_phase(XI(s, b, i, j), ZI(s, b, i, j), XI(s, b, k, j), ZI(s, b, k, j));
    int32_t p = (int32_t)((((sum % 4) + 4) % 4) >> 1);
    return RI(s, b, i) ^ RI(s, b, k) ^ p;
}

/* RowMultiply (MeasurementFunctors.hpp:156-166). */
static void row_multiply(ora_state *s, int64_t b, int64_t i, int64_t k) {
    RI(s, b, i) = row_product_sign(s, b, i, k);
    for (int64_t j = 0; j < s->n; ++j) {
        XI(s, b, i, j) ^= XI(s, b, k, j);
        ZI(s, b, i, j) ^= ZI(s, b, k, j);
    }
}

/* ZeroRow (MeasurementFunctors.hpp:86-95). */
static void zero_row(ora_state *s, int64_t b, int64_t row) {
    for (int64_t j = 0; j < s->n; ++j) {
        XI(s, b, row, j) = 0;
        ZI(s, b, row, j) = 0;
    }
    RI(s, b, row) = 0;
}

/* CopyFromRowAtoRowB (MeasurementFunctors.hpp:74-84). */
static void copy_row(ora_state *s, int64_t b, int64_t from, int64_t to) {
    for (int64_t j = 0; j < s->n; ++j) {
        XI(s, b, to, j) = XI(s, b, from, j);
        ZI(s, b, to, j) = ZI(s, b, from, j);
    }
    RI(s, b, to) = RI(s, b, from);
}

/* MeasureDetermined (MeasurementFunctors.hpp:189-201). */
static int32_t measure_determined(ora_state *s, int64_t b, int64_t q) {
    const int64_t n = s->n;
    zero_row(s, b, 2 * n);
    for (int64_t i = 0; i < n; ++i)
        if (XI(s, b, i, q)) row_multiply(s, b, 2 * n, i + n);
    return RI(s, b, 2 * n);
}

static int forced_bit(const uint8_t *forced, int64_t shot) { return (forced[shot >> 3] >> (shot & 7)) & 1; }

/* MeasureRandom (MeasurementFunctors.hpp:225-265).  The outcome replaces
 * `frand(0,1) < bias` with a forced bit or a Philox draw. */
static int32_t measure_random(ora_state *s, int64_t b, int64_t q, int64_t p, float bias, uint64_t event,
                              const uint8_t *forced) {
    const int64_t n = s->n;
    copy_row(s, b, p + n, p);
    zero_row(s, b, p + n);
    ZI(s, b, p + n, q) = 1;
    /* A forced bit stands for the draw 0.25 (bit 1) or 0.75 (bit 0), so at
     * the default bias 0.5 the outcome is the bit and bias 0 / 1 still force
     * 0 / 1, as the reference's `frand < bias` does. */
    float u = forced ? (forced_bit(forced, b) ? 0.25f : 0.75f)
                     : u32_to_unit_float(ora_draw_u32(s->seed, event, s->shot_base + b, TAG_MEASURE));
    RI(s, b, p + n) = u < bias;
    for (int64_t i = 0; i < 2 * n; ++i)
        if (XI(s, b, i, q) && i != p && i != p + n) row_multiply(s, b, i, p);
    return RI(s, b, p + n);
}

static ora_record *new_record(ora_state *s, int64_t q) {
    if (s->nrecs == s->caprecs) {
        s->caprecs = s->caprecs ? 2 * s->caprecs : 16;
        s->recs = (ora_record *)realloc(s->recs, (size_t)s->caprecs * sizeof(ora_record));
    }
    ora_record *rec = &s->recs[s->nrecs++];
    rec->qubit = q;
    rec->res = (int32_t *)calloc((size_t)(s->batch ? s->batch : 1), sizeof(int32_t));
    rec->det = (int32_t *)calloc((size_t)(s->batch ? s->batch : 1), sizeof(int32_t));
    return rec;
}

/* MeasureQubit (CliffordState.hpp:587-623) + BatchMeasureFunctor
 * (MeasurementFunctors.hpp:291-317): per shot, the lowest stabilizer row
 * p+n with x(p+n,q)=1 selects the random branch, else deterministic. */
int64_t ora_measure(ora_state *s, int64_t q, float bias, int64_t id, const uint8_t *forced) {
    int64_t rid;
    if (id < 0) {
        new_record(s, q);
        rid = s->nrecs - 1;
    } else {
        if (id >= s->nrecs) return -1; /* CliffordState.hpp:609-610 */
        rid = id;
    }
    ora_record *rec = &s->recs[rid];
    const uint64_t event = s->events++;
    const int64_t n = s->n;
#pragma omp parallel for num_threads(OMP_THREADS()) schedule(static)
    for (int64_t b = 0; b < s->batch; ++b) {
        int64_t p;
        for (p = 0; p < n; ++p)
            if (XI(s, b, p + n, q)) break;
        if (p < n) {
            rec->res[b] = measure_random(s, b, q, p, bias, event, forced);
            rec->det[b] = 0;
        } else {
            rec->res[b] = measure_determined(s, b, q);
            rec->det[b] = 1;
        }
    }
    return rid;
}

int64_t ora_reset_qubit(ora_state *s, int64_t q, const uint8_t *forced) {
    int64_t rid = ora_measure(s, q, 0.5f, -1, forced);
    const int32_t *flag = s->recs[rid].res;
    /* Conditional X = H S S H, each with the record as apply flag
     * (the composition Test_CliffordState.hpp:703-711 uses). */
    ora_h_flag(s, q, flag);
    ora_s_flag(s, q, flag);
    ora_s_flag(s, q, flag);
    ora_h_flag(s, q, flag);
    return rid;
}

int64_t ora_num_records(const ora_state *s) { return s->nrecs; }

/* GetMeasurement(id, shot) (CliffordState.hpp:635-648). */
int ora_get_measurement(const ora_state *s, int64_t id, int64_t shot, int32_t *res, int32_t *det) {
    if (id < 0 || id >= s->nrecs || shot < 0 || shot >= s->batch) return -1;
    *res = s->recs[id].res[shot];
    *det = s->recs[id].det[shot];
    return 0;
}
const int32_t *ora_record_results(const ora_state *s, int64_t id) { return s->recs[id].res; }
const int32_t *ora_record_determined(const ora_state *s, int64_t id) { return s->recs[id].det; }
int64_t ora_record_qubit(const ora_state *s, int64_t id) { return s->recs[id].qubit; }

/* -------------------------------------------------------------- noise */
/* Pauli index 0..3 = I, X, Y, Z.  X or Y flips signs of rows with z_q
 * (conditional X = H S S H with flag), Y or Z flips rows with x_q
 * (conditional Z = S S with flag). */
static void apply_flag_paulis(ora_state *s, int64_t q, const int32_t *fx, const int32_t *fz) {
    ora_h_flag(s, q, fx);
    ora_s_flag(s, q, fx);
    ora_s_flag(s, q, fx);
    ora_h_flag(s, q, fx);
    ora_s_flag(s, q, fz);
    ora_s_flag(s, q, fz);
}

/* Pauli-channel sampling (this library's own scheme; the reference has no
 * channel op).  thr[k] = ora_threshold of the cumulative probability of
 * Paulis 1..k+1, total = thr[count-1]: a shot is hit with probability
 * total / 2^32 and a hit takes Pauli k+1 with probability
 * (thr[k] - thr[k-1]) / total.  The 64 shots of a global word are sampled by
 * gaps: with S_0 = 2^32 and S_{j+1} = floor(S_j (2^32 - total) / 2^32), a
 * draw u puts the next hit g shots on, g the first with u >= S_{g+1}; one
 * more draw v picks the hit's Pauli, the first k with
 * floor(v total / 2^32) < thr[k].  The first draw of a word is lane
 * event%4 of Philox block (0, word, event/4, TAG_NOISE_FIRST) -- one block
 * serves four consecutive channel events -- and draw i >= 1 is lane
 * (i-1)%4 of block (1 + (i-1)/4, word, event, TAG_NOISE). */
static uint64_t surv64(uint64_t total) {
    if (total == 0) return (uint64_t)1 << 32;
    const uint64_t q = ((uint64_t)1 << 32) - total;
    uint64_t s = (uint64_t)1 << 32;
    for (int j = 0; j < 64; ++j) s = (s * q) >> 32;
    return s;
}

static void channel_word(int64_t seed, uint64_t event, uint64_t word, const uint64_t *thr, int count, uint64_t s64,
                         int32_t idx[64]) {
    memset(idx, 0, 64 * sizeof(int32_t));
    const uint64_t total = thr[count - 1];
    if (total == 0) return;
    const uint32_t key[2] = {(uint32_t)((uint64_t)seed & 0xffffffffu), (uint32_t)((uint64_t)seed >> 32)};
    uint32_t ctr[4] = {0u, (uint32_t)word, (uint32_t)(event >> 2), TAG_NOISE_FIRST}, blk[4];
    ora_philox4x32_10(ctr, key, blk);
    uint32_t u = blk[event & 3u];
    if ((uint64_t)u < s64) return;
    const uint64_t q = ((uint64_t)1 << 32) - total;
    ctr[2] = (uint32_t)event;
    ctr[3] = TAG_NOISE;
    uint32_t i = 0; /* later draws: lane i%4 of block 1 + i/4 */
    int pos = 0;
    for (;;) {
        uint64_t s = (uint64_t)1 << 32;
        for (;;) {
            s = (s * q) >> 32;
            if ((uint64_t)u >= s) break;
            if (++pos == 64) return;
        }
        if ((i & 3u) == 0u) {
            ctr[0] = 1u + (i >> 2);
            ora_philox4x32_10(ctr, key, blk);
        }
        const uint64_t v = ((uint64_t)blk[i & 3u] * total) >> 32;
        ++i;
        int k = 1;
        while (v >= thr[k - 1]) ++k;
        idx[pos] = k;
        if (++pos == 64) return;
        if ((i & 3u) == 0u) {
            ctr[0] = 1u + (i >> 2);
            ora_philox4x32_10(ctr, key, blk);
        }
        u = blk[i & 3u];
        ++i;
    }
}

void ora_channel_paulis(int64_t seed, uint64_t event, int64_t shot_base, int64_t batch, const float *p, int count,
                        int32_t *out) {
    uint64_t thr[15];
    double cum = 0.0;
    for (int k = 0; k < count; ++k) {
        cum += (double)p[k];
        thr[k] = ora_threshold(cum);
    }
    const uint64_t s64 = surv64(thr[count - 1]);
    int32_t idx[64];
    int64_t cur = -1;
    for (int64_t b = 0; b < batch; ++b) {
        const int64_t g = shot_base + b;
        if ((g >> 6) != cur) {
            cur = g >> 6;
            channel_word(seed, event, (uint64_t)cur, thr, count, s64, idx);
        }
        out[b] = idx[g & 63];
    }
}

void ora_pauli_channel_1(ora_state *s, int64_t q, const float p[3]) {
    const uint64_t event = s->events++;
    int32_t *k = (int32_t *)calloc((size_t)s->batch + 1, sizeof(int32_t));
    int32_t *fx = (int32_t *)calloc((size_t)s->batch + 1, sizeof(int32_t));
    int32_t *fz = (int32_t *)calloc((size_t)s->batch + 1, sizeof(int32_t));
    ora_channel_paulis(s->seed, event, s->shot_base, s->batch, p, 3, k);
    for (int64_t b = 0; b < s->batch; ++b) {
        fx[b] = (k[b] == 1 || k[b] == 2);
        fz[b] = (k[b] == 2 || k[b] == 3);
    }
    apply_flag_paulis(s, q, fx, fz);
    free(k);
    free(fx);
    free(fz);
}

void ora_pauli_channel_2(ora_state *s, int64_t a, int64_t bq, const float p[15]) {
    const uint64_t event = s->events++;
    size_t sz = (size_t)s->batch + 1;
    int32_t *k = (int32_t *)calloc(sz, 4);
    int32_t *fxa = (int32_t *)calloc(sz, 4), *fza = (int32_t *)calloc(sz, 4);
    int32_t *fxb = (int32_t *)calloc(sz, 4), *fzb = (int32_t *)calloc(sz, 4);
    ora_channel_paulis(s->seed, event, s->shot_base, s->batch, p, 15, k);
    for (int64_t b = 0; b < s->batch; ++b) {
        int pa = k[b] >> 2, pb = k[b] & 3;
        fxa[b] = (pa == 1 || pa == 2);
        fza[b] = (pa == 2 || pa == 3);
        fxb[b] = (pb == 1 || pb == 2);
        fzb[b] = (pb == 2 || pb == 3);
    }
    apply_flag_paulis(s, a, fxa, fza);
    apply_flag_paulis(s, bq, fxb, fzb);
    free(k);
    free(fxa);
    free(fza);
    free(fxb);
    free(fzb);
}

/* -------------------------------------------------------------- circuits */
int ora_run(ora_state *s, const ora_op *ops, int64_t nops, const float *params, const uint8_t *forced_all) {
    const size_t fbytes = (size_t)((s->batch + 7) / 8);
    int64_t kmeas = 0;
    for (int64_t k = 0; k < nops; ++k) {
        const ora_op *o = &ops[k];
        const uint8_t *forced = forced_all ? forced_all + (size_t)kmeas * fbytes : NULL;
        switch (o->code) {
        case ORA_OP_H: ora_h(s, o->a); break;
        case ORA_OP_S: ora_s(s, o->a); break;
        case ORA_OP_X: ora_x_gate(s, o->a); break;
        case ORA_OP_Y: ora_y_gate(s, o->a); break;
        case ORA_OP_Z: ora_z_gate(s, o->a); break;
        case ORA_OP_CX: ora_cx(s, o->a, o->b); break;
        case ORA_OP_CZ: ora_cz(s, o->a, o->b); break;
        case ORA_OP_M:
            ora_measure(s, o->a, o->c >= 0 ? params[o->c] : 0.5f, -1, forced);
            ++kmeas;
            break;
        case ORA_OP_R:
            ora_reset_qubit(s, o->a, forced);
            ++kmeas;
            break;
        case ORA_OP_PAULI1: ora_pauli_channel_1(s, o->a, params + o->c); break;
        case ORA_OP_PAULI2: ora_pauli_channel_2(s, o->a, o->b, params + o->c); break;
        case ORA_OP_H_IF:
            if (o->c < 0 || o->c >= s->nrecs) return -1;
            ora_h_flag(s, o->a, s->recs[o->c].res);
            break;
        case ORA_OP_S_IF:
            if (o->c < 0 || o->c >= s->nrecs) return -1;
            ora_s_flag(s, o->a, s->recs[o->c].res);
            break;
        default: return -1;
        }
    }
    return 0;
}

/* ------------------------------------------------------------ test hooks */
/* BatchRowProductSignFunctor / BatchRowMultiplyFunctor /
 * BatchMeasureDeterminedFunctor (MeasurementFunctors.hpp:132-187, :344-364). */
int32_t ora_row_product_sign(const ora_state *s, int64_t shot, int64_t i, int64_t k) {
    return row_product_sign(s, shot, i, k);
}
void ora_row_multiply(ora_state *s, int64_t shot, int64_t i, int64_t k) { row_multiply(s, shot, i, k); }
int32_t ora_measure_determined(ora_state *s, int64_t shot, int64_t q) { return measure_determined(s, shot, q); }
