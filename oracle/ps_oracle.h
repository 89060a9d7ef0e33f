/*
 * ps_oracle.h -- CPU oracle for the batched stabilizer-tableau path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a restatement, in plain C, of the
 * reference's CliffordState algorithm (plaquette_simulator/src/
 * CliffordState.hpp, GateFunctors.hpp, MeasurementFunctors.hpp,
 * MiscFunctors.hpp) in the reference's own storage layout: one int32 per
 * tableau bit, row-major [shot][row][qubit] with W = 2n+1 rows (row 2n is the
 * scratch row).  It is used by the tests as the parity checker, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline / reference arm.
 * The product (the CUDA library) never links or calls it.
 *
 * Parity pinning: the restatement is checked against the reference's own
 * golden vectors (Test_CliffordState.hpp) and, where the reference headers are
 * available, against the unmodified reference compiled on a Kokkos-API shim
 * (oracle/_ref).
 *
 * Randomness: random measurement outcomes are either forced from a caller bit
 * table (the same bit table the reference build consumes through its shim) or
 * drawn from Philox4x32-10 keyed by (seed, event index, global shot).  Pauli
 * noise channels are drawn from the same generator.  Both are restated in
 * ps_oracle.c from the published algorithm, independently of the CUDA code.
 */
#ifndef PS_ORACLE_H
#define PS_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_state ora_state;

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11). */
void ora_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Construction mirrors CliffordState(n, batch, seed, init_to_zero)
 * (CliffordState.hpp:97-139).  shot_base is the global index of local shot 0,
 * so a sub-range of a large batch can be replayed shot-for-shot. */
ora_state *ora_create(int64_t n, int64_t batch, int64_t seed, int init_zero, int64_t shot_base);
ora_state *ora_create_from_host(const int32_t *x, const int32_t *z, const int32_t *r,
                                int64_t n, int64_t batch, int64_t seed, int64_t shot_base);
ora_state *ora_clone(const ora_state *s);
void ora_destroy(ora_state *s);

int64_t ora_num_qubits(const ora_state *s);
int64_t ora_batch(const ora_state *s);
int64_t ora_seed(const ora_state *s);
uint64_t ora_events(const ora_state *s);
void ora_set_threads(int nthreads);

/* Reference int layout views: x,z are [batch][2n+1][n], r is [batch][2n+1]. */
void ora_device_to_host(const ora_state *s, int32_t *x, int32_t *z, int32_t *r);
void ora_host_to_device(ora_state *s, const int32_t *x, const int32_t *z, const int32_t *r);
int32_t *ora_x(ora_state *s);
int32_t *ora_z(ora_state *s);
int32_t *ora_r(ora_state *s);

void ora_reset(ora_state *s); /* intended semantics of ResetCliffordState */
int64_t ora_checksum(const ora_state *s, int64_t s0, int64_t s1);

/* Gates (GateFunctors.hpp). */
void ora_h(ora_state *s, int64_t q);
void ora_s(ora_state *s, int64_t q);
void ora_x_gate(ora_state *s, int64_t q);
void ora_y_gate(ora_state *s, int64_t q);
void ora_z_gate(ora_state *s, int64_t q);
void ora_cx(ora_state *s, int64_t c, int64_t t);
void ora_cz(ora_state *s, int64_t c, int64_t t);
/* WithApplyFlag forms; flag = a per-shot int32 array (a measurement record). */
void ora_h_flag(ora_state *s, int64_t q, const int32_t *flag);
void ora_s_flag(ora_state *s, int64_t q, const int32_t *flag);

/* MeasureQubit (CliffordState.hpp:587-623).  id < 0 allocates a new record.
 * forced: packed bits, LSB-first, ceil(batch/8) bytes, or NULL for Philox.
 * A forced bit stands for the uniform draw 0.25 (bit 1) or 0.75 (bit 0);
 * the outcome is draw < bias.  Returns the record id, or -1 if id is out of
 * range. */
int64_t ora_measure(ora_state *s, int64_t q, float bias, int64_t id, const uint8_t *forced);
/* ResetQubit: MeasureQubit into a new record, then conditional X (as the
 * reference composes it: H,S,S,H with the record as apply flag). */
int64_t ora_reset_qubit(ora_state *s, int64_t q, const uint8_t *forced);
int64_t ora_num_records(const ora_state *s);
/* 0 ok, -1 out of range (the reference's nullopt). */
int ora_get_measurement(const ora_state *s, int64_t id, int64_t shot, int32_t *res, int32_t *det);
const int32_t *ora_record_results(const ora_state *s, int64_t id);
const int32_t *ora_record_determined(const ora_state *s, int64_t id);
int64_t ora_record_qubit(const ora_state *s, int64_t id);

/* Pauli channels.  p = 3 probabilities (X, Y, Z) or 15 probabilities for
 * the two-qubit Paulis in order IX IY IZ XI XX XY XZ YI YX YY YZ ZI ZX ZY ZZ
 * (first letter on qubit a).  Applied as conditional X / Z through the
 * reference's flag gates. */
void ora_pauli_channel_1(ora_state *s, int64_t q, const float p[3]);
void ora_pauli_channel_2(ora_state *s, int64_t a, int64_t b, const float p[15]);

/* Circuit op records (same encoding as the product's ps_op). */
typedef struct {
    int32_t code, a, b, c;
} ora_op;
enum {
    ORA_OP_H = 0, ORA_OP_S = 1, ORA_OP_X = 2, ORA_OP_Y = 3, ORA_OP_Z = 4,
    ORA_OP_CX = 5, ORA_OP_CZ = 6, ORA_OP_M = 7, ORA_OP_R = 8,
    ORA_OP_PAULI1 = 9, ORA_OP_PAULI2 = 10, ORA_OP_H_IF = 11, ORA_OP_S_IF = 12
};
/* Runs ops in order; params holds channel probabilities / biases (c indexes
 * it; for M/R, c < 0 means bias 0.5).  H_IF / S_IF take c = record id.
 * forced_all: for the k-th measurement (M or R) of the run, bits at
 * forced_all + k * ceil(batch/8), or NULL.  Returns 0 or -1 on a bad op. */
int ora_run(ora_state *s, const ora_op *ops, int64_t nops, const float *params,
            const uint8_t *forced_all);

/* Threshold used for Pauli-channel sampling: u32 < T means "inside". */
uint64_t ora_threshold(double cumulative);
/* The Pauli a channel event puts on shots [shot_base, shot_base + batch):
 * out[b] = 0 (identity) or the index into p plus 1, drawn word by word by
 * the gap sampling described in ps_oracle.c. */
void ora_channel_paulis(int64_t seed, uint64_t event, int64_t shot_base, int64_t batch, const float *p, int count,
                        int32_t *out);
/* One 32-bit Philox draw for (seed, event, global shot, tag); tag 1 =
 * measurement outcome, 2 = Pauli channel. */
uint32_t ora_draw_u32(int64_t seed, uint64_t event, int64_t gshot, uint32_t tag);

/* Test hooks for the reference's test-only functors. */
int32_t ora_row_product_sign(const ora_state *s, int64_t shot, int64_t i, int64_t k);
void ora_row_multiply(ora_state *s, int64_t shot, int64_t i, int64_t k);
int32_t ora_measure_determined(ora_state *s, int64_t shot, int64_t q);
int32_t ora_pauli_product_phase(int32_t x1, int32_t z1, int32_t x2, int32_t z2);

#ifdef __cplusplus
}
#endif
#endif
