/*
 * plaquette_gpu.h -- C ABI of the GB300 batched stabilizer-tableau library
 * (libps_gpu.so).
 *
 * It is a drop-in for the state API of the reference,
 * Plaquette::CliffordState<int> (plaquette_simulator/src/CliffordState.hpp)
 * and its Python binding (plaquette_simulator/src/Bindings.cpp:13-31).  Each
 * entry point below names the reference interface it replaces.  All compute
 * runs in hand-written sm_103a CUDA kernels; there is no CPU fallback.
 *
 * Conventions
 *  - Every call returns a ps_status (PS_OK = 0).  On error, ps_last_error()
 *    returns a thread-local message in the reference's error format
 *    (Error.hpp:94-97: "[file][Line:N][Method:f]: Error in Plaquette: msg").
 *  - A handle owns its device tableau, its measurement records and one CUDA
 *    stream.  Calls that return host data synchronise that stream (the
 *    reference's deep_copy is blocking too).  One handle must not be used from
 *    several host threads at once (as in the reference, whose measurement
 *    list is unsynchronised, CliffordState.hpp:593).
 *  - Host tableau buffers use the reference's int32 layout: x and z are
 *    [batch][2n+1][n], r is [batch][2n+1], row-major
 *    (CliffordState.hpp:207-259).
 *  - Random measurement outcomes: `forced` is NULL (per-shot Philox4x32-10
 *    draws keyed by (seed, event index, global shot)) or ceil(batch/8) bytes
 *    of LSB-first bits; a forced bit stands for the uniform draw 0.25 (bit 1)
 *    or 0.75 (bit 0), and the outcome is draw < bias, as `frand(0,1) < bias`
 *    in MeasurementFunctors.hpp:245-247.
 */
#ifndef PLAQUETTE_GPU_H
#define PLAQUETTE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ps_status;
#define PS_OK 0
#define PS_E_ARG 1     /* invalid argument (qubit out of range, bad size ...) */
#define PS_E_RANGE 2   /* id/shot out of range; GetMeasurement's nullopt     */
#define PS_E_CUDA 3    /* CUDA runtime error                                 */
#define PS_E_NOMEM 4   /* device allocation failed / over budget             */
#define PS_E_STATE 5   /* call not valid in the handle's current state       */
#define PS_E_TIMEOUT 6 /* a bounded device wait gave up                      */

typedef struct ps_state ps_state;

/* Thread-local message of the last failed call ("" if none). */
const char *ps_last_error(void);
/* Replaces CliffordState::GetKokkosBackend (CliffordState.hpp:280-282):
 * "CUDA sm_103a (<device name>)". */
const char *ps_backend_name(void);
/* Library version string. */
const char *ps_version(void);
/* Selects the CUDA device used by handles created afterwards on the calling
 * thread (one process per GPU). */
ps_status ps_set_device(int device);
/* Waits for all work of this library on the current device (also run
 * automatically at process exit, before the CUDA runtime shuts down). */
ps_status ps_device_synchronize(void);

/* ---------------------------------------------------------------- state */
/* CliffordState(num_qubits, batch_size, seed = -1, init_to_zero_state)
 * (CliffordState.hpp:97-139).  seed < 0 falls back to 213434232223 as there. */
ps_status ps_create(uint64_t num_qubits, uint64_t batch_size, int64_t seed, int init_to_zero_state,
                    ps_state **out);
/* CliffordState(x, z, r, num_qubits, batch_size, seed) (CliffordState.hpp:153-159). */
ps_status ps_create_from_host(const int32_t *x, const int32_t *z, const int32_t *r, uint64_t num_qubits,
                              uint64_t batch_size, int64_t seed, ps_state **out);
/* Copy constructor (CliffordState.hpp:168-174): tableau, seed and event
 * counter are copied; measurement records are not (as in the reference). */
ps_status ps_clone(const ps_state *h, ps_state **out);
/* ~CliffordState (CliffordState.hpp:665-688).  NULL is a no-op. */
ps_status ps_destroy(ps_state *h);

ps_status ps_get_num_qubits(const ps_state *h, uint64_t *out); /* GetNumQubits :289 */
ps_status ps_get_batch_size(const ps_state *h, uint64_t *out); /* GetBatchSize :296 */
ps_status ps_get_seed(const ps_state *h, int64_t *out);        /* GetSeed :303      */
/* Number of random events (measurements and Pauli channels) consumed so far;
 * the next one draws with this event index. */
ps_status ps_get_event_counter(const ps_state *h, uint64_t *out);
ps_status ps_set_event_counter(ps_state *h, uint64_t events);
/* The global index of the state's first shot (a multiple of 64; default 0).
 * Random draws are keyed by global shot, so one job's shots split over
 * several states -- e.g. one per GPU, shots [r*S, (r+1)*S) on rank r -- give
 * exactly the records of one state holding all of them.  No counterpart in
 * the reference (one state per job). */
ps_status ps_set_shot_offset(ps_state *h, uint64_t first_shot);
ps_status ps_get_shot_offset(const ps_state *h, uint64_t *first_shot);

/* ResetCliffordState (CliffordState.hpp:309-316).  Implements the intended
 * semantics (the tableau of a fresh constructor); the reference's launch
 * policy {B, W, W} writes out of bounds. */
ps_status ps_reset(ps_state *h);
/* CheckSum(starting_batch_id, ending_batch_id) (CliffordState.hpp:327-338):
 * sum of all x, z, r entries of shots [s0, s1); s1 < 0 means batch_size. */
ps_status ps_checksum(ps_state *h, int64_t s0, int64_t s1, int64_t *out);
/* DeviceToHost / HostToDevice (CliffordState.hpp:207-259), reference layout. */
ps_status ps_device_to_host(ps_state *h, int32_t *x, int32_t *z, int32_t *r);
ps_status ps_host_to_device(ps_state *h, const int32_t *x, const int32_t *z, const int32_t *r);

/* ---------------------------------------------------------------- gates */
/* Apply{Hadamard,Phase,PauliX,PauliY,PauliZ}Gate (CliffordState.hpp:389-531). */
ps_status ps_h(ps_state *h, uint64_t q);
ps_status ps_s(ps_state *h, uint64_t q);
ps_status ps_x(ps_state *h, uint64_t q);
ps_status ps_y(ps_state *h, uint64_t q);
ps_status ps_z(ps_state *h, uint64_t q);
/* ApplyControlNotGate / ApplyControlPhaseGate (CliffordState.hpp:412-449). */
ps_status ps_cx(ps_state *h, uint64_t control, uint64_t target);
ps_status ps_cz(ps_state *h, uint64_t control, uint64_t target);
/* Apply*GateToQubits (CliffordState.hpp:379-531): one gate per target (per
 * consecutive pair for CX / CZ). */
ps_status ps_apply_to_qubits(ps_state *h, int32_t op_code, const uint64_t *targets, uint64_t count);
/* Apply{Hadamard,Phase}GateWithApplyFlag (CliffordState.hpp:348-372); the
 * apply flag is the result array of measurement record `meas_id` (the
 * reference passes that record's device View). */
ps_status ps_h_flag(ps_state *h, uint64_t q, uint64_t meas_id);
ps_status ps_s_flag(ps_state *h, uint64_t q, uint64_t meas_id);

/* ---------------------------------------------------------- measurement */
/* MeasureQubit(target_qubit, bias, measurement_id) (CliffordState.hpp:587-623).
 * id < 0 creates a new record; an existing id is overwritten (the
 * reference's "Measurement id is out of range" check at :609-610 becomes
 * PS_E_RANGE).  *out_id receives the record id. */
ps_status ps_measure(ps_state *h, uint64_t q, float bias, int64_t id, const uint8_t *forced, uint64_t *out_id);
/* MeasureQubits(targets, bias) (CliffordState.hpp:543-548): one record per
 * target; ids are consecutive starting at *first_id. */
ps_status ps_measure_qubits(ps_state *h, const uint64_t *targets, uint64_t count, float bias,
                            uint64_t *first_id);
/* GetMeasurement(id, shot) (CliffordState.hpp:635-648): PS_E_RANGE where the
 * reference returns nullopt. */
ps_status ps_get_measurement(ps_state *h, uint64_t id, uint64_t shot, int32_t *result, int32_t *determined);
/* All shots of one record, bit-packed LSB-first (ceil(batch/8) bytes each;
 * either pointer may be NULL). */
ps_status ps_get_record_bits(ps_state *h, uint64_t id, uint8_t *result_bits, uint8_t *determined_bits);
ps_status ps_num_records(const ps_state *h, uint64_t *out);
/* Qubit that record `id` measured (Measurement::qubit_measured, :33). */
ps_status ps_record_qubit(const ps_state *h, uint64_t id, uint64_t *out);

/* --------------------------------------------------- ops with no counterpart */
/* ResetQubit: MeasureQubit into a new record, then X on the shots whose
 * outcome is 1 (the reference composes that X as H,S,S,H with the record as
 * apply flag, Test_CliffordState.hpp:703-711). */
ps_status ps_reset_qubit(ps_state *h, uint64_t q, const uint8_t *forced, uint64_t *out_id);
/* Pauli channel on q: per shot X / Y / Z with probabilities p[0..2], drawn
 * from Philox keyed by (seed, event index, shot).  Mirrors the E_PAULI
 * parameter count of CliffordCircuit.hpp:44-49. */
ps_status ps_pauli_channel_1(ps_state *h, uint64_t q, const float p[3]);
/* Two-qubit Pauli channel on (a, b); p[15] in the order IX IY IZ XI XX XY XZ
 * YI YX YY YZ ZI ZX ZY ZZ.  Mirrors E_PAULI2 (CliffordCircuit.hpp:50-55). */
ps_status ps_pauli_channel_2(ps_state *h, uint64_t a, uint64_t b, const float p[15]);

/* Same channel and random draws as ps_pauli_channel_1, for callers that must
 * not allocate device memory during the call (a host that has already handed
 * the whole device to its own memory pool, a process under a strict memory
 * budget, or code that must not risk the device-wide synchronisation an
 * allocation can cause).  It has no counterpart in the reference.  Its scratch
 * is a fixed 258 KiB array inside the library: at most 524,288 shots (8,192
 * shot-words) per state, larger states get PS_E_ARG.  The first call on a
 * device looks up that array's address and must not be made while a stream is
 * being captured; calls on different streams that overlap on the GPU share
 * the array and race. */
ps_status ps_pauli_channel_1_noalloc(ps_state *h, uint64_t q, const float p[3]);

/* ------------------------------------------------------------- circuits */
/* A circuit is an op table (see the PS_OP_* codes) plus a float parameter
 * table.  It replaces the reference's CliffordCircuit driver
 * (CliffordCircuit.hpp:131-135, one parallel_for per target) with a compiled
 * plan bound to one state:
 *   PS_MODE_PLAIN  one kernel launch per op (the reference's structure);
 *   PS_MODE_FUSED  every run of gates / Pauli gates / channels / reset-X
 *                  between measurement phases is one fused pass over the
 *                  tableau; each run of consecutive measurements is one
 *                  launch.
 * With use_graph the whole plan is captured once into a CUDA graph and each
 * run is one graph launch. */
typedef struct {
    int32_t code, a, b, c;
} ps_op;
#define PS_OP_H 0
#define PS_OP_S 1
#define PS_OP_X 2
#define PS_OP_Y 3
#define PS_OP_Z 4
#define PS_OP_CX 5      /* a = control, b = target                           */
#define PS_OP_CZ 6
#define PS_OP_M 7       /* bias = params[c] (c < 0: 0.5)                      */
#define PS_OP_R 8       /* measure into a record, then X where the outcome is 1 */
#define PS_OP_PAULI1 9  /* params[c..c+2] = pX, pY, pZ                        */
#define PS_OP_PAULI2 10 /* params[c..c+14], order IX IY ... ZZ                 */
#define PS_OP_H_IF 11   /* H on a where circuit record c (k-th M/R) is 1       */
#define PS_OP_S_IF 12

#define PS_MODE_PLAIN 0
#define PS_MODE_FUSED 1

typedef struct {
    int32_t mode;        /* PS_MODE_PLAIN or PS_MODE_FUSED                      */
    int32_t use_graph;   /* capture the plan in a CUDA graph                     */
    int32_t seg_rows;    /* fused tile: tableau rows per CTA (0 = auto)          */
    int32_t seg_words;   /* fused tile: 64-shot words per CTA (0 = auto)         */
    int32_t seg_threads; /* fused tile: threads per CTA (0 = auto)               */
    int32_t meas_words;  /* measurement kernel: shot-words per CTA, 1, 2 or 4 (0 = auto) */
    int32_t seg_resident; /* fused segments: 0 = one warp per (row, shot-word),
                             every gate through shared memory; 1 = keep
                             gate-dense columns in registers where possible
                             (channel outcomes and sign ops then act after the
                             last layer through propagated Paulis); 2 = one
                             thread per gate over all shot-words of a one-row
                             tile                                             */
    int32_t per_shot_xz; /* fused runs from |0...0>: 0 = share the x / z bits of
                             all shots and run a sign program when the circuit
                             has no per-shot conditional gate (H_IF / S_IF):
                             bit-identical, and the final x / z bits are
                             written to every shot; 1 = always update every
                             shot's tableau                                   */
    int32_t frame_warps; /* shared-x/z runs: sign-kernel warps per shot-word, 4
                             or 8 (0 = auto)                                  */
    int32_t bcast_ctas;  /* shared-x/z runs: x / z broadcast CTAs (8 warps)
                             per SM (0 = auto: 1); the rest of each SM runs
                             the noise and sign kernels                       */
} ps_circuit_options;

typedef struct {
    uint64_t num_ops, num_gates, num_measurements, num_channels, num_events;
    uint64_t num_segments, num_measure_phases, launches_per_run;
    uint64_t first_record;          /* state record id of the first M/R      */
    double segment_bytes;           /* algorithmic HBM bytes of all segments  */
    int32_t seg_rows, seg_words, seg_threads, meas_words;
    int32_t resident_segments;      /* segments in the register-resident form */
    int32_t shared_xz;              /* 1: runs from |0...0> use the shared-x/z plan */
    int32_t frame_warps, bcast_ctas; /* shared-x/z knobs in use (sign-kernel warps
                                        per shot-word, broadcast CTAs per SM) */
    int32_t pad;
} ps_circuit_stats;

typedef struct ps_circuit ps_circuit;

/* Compiles ops for state h; allocates one measurement record per M / R (ids
 * first_record .. first_record + num_measurements - 1). */
ps_status ps_circuit_compile(ps_state *h, const ps_op *ops, uint64_t nops, const float *params, uint64_t nparams,
                             const ps_circuit_options *opts, ps_circuit **out);
/* The compile cache (no counterpart in the reference): the shot-independent
 * host work of ps_circuit_compile -- segment schedules, the measurement
 * plan, the shared-x/z sign program -- is kept per process for the most
 * recent 128 distinct (qubit count, options, op table, parameter table)
 * keys, so a circuit compiled again (a served or batched job of a shape seen
 * before) only allocates, uploads and captures.  Counts since the last
 * clear; any pointer may be NULL. */
ps_status ps_compile_cache_stats(uint64_t *hits, uint64_t *misses, uint64_t *entries);
ps_status ps_compile_cache_clear(void);
/* Forced random draws for the circuit's measurements: num_measurements rows
 * of ceil(batch/8) bytes, or NULL to return to Philox draws. */
ps_status ps_circuit_set_forced(ps_circuit *c, const uint8_t *forced_all);
/* Enqueues one run on the state's stream (returns without waiting).  The run
 * draws with event indices starting at the state's event counter, which it
 * advances by num_events.  reset_state != 0 first re-initialises the tableau
 * to |0...0> (inside the same graph). */
ps_status ps_circuit_run(ps_circuit *c, int reset_state);
ps_status ps_circuit_get_stats(const ps_circuit *c, ps_circuit_stats *out);
ps_status ps_circuit_destroy(ps_circuit *c);

/* Per-kernel-kind device time of one run, measured with CUDA events around
 * every launch (the plan is enqueued launch by launch, not as a graph, and
 * the call waits for it).  Kinds: 0 tableau init, 1 channel sampling (fused),
 * 2 fused segment, 3 measurement, 4 per-op gate, 5 per-op channel, 6 sign
 * program (shared x/z), 7 x / z broadcast (shared x/z). */
#define PS_PROFILE_KINDS 8
typedef struct {
    double ms[PS_PROFILE_KINDS];
    uint64_t launches[PS_PROFILE_KINDS];
} ps_circuit_profile_t;
ps_status ps_circuit_profile(ps_circuit *c, int reset_state, ps_circuit_profile_t *out);
/* Runs the circuit once (launch by launch) and reports, for each of its
 * measurements in order and for shots 0..63, whether the random branch was
 * taken and how many tableau rows were multiplied.  Used to count the
 * algorithmic bytes of the measurement phases. */
ps_status ps_circuit_measure_stats(ps_circuit *c, int reset_state, int32_t *random_branch, int32_t *rows);
/* Copies the results / determined words of every record of the circuit to
 * host memory: num_measurements rows of `words` uint64 each (bit s of word
 * k = shot 64k+s).  Either pointer may be NULL.  Waits for the stream. */
ps_status ps_circuit_copy_records(ps_circuit *c, uint64_t *results, uint64_t *determined, uint64_t *words);
/* Pipelined sampling (no counterpart in the reference): enqueues the copy of
 * the records of c's latest run to host memory on copy_stream (a
 * cudaStream_t as void*; NULL = a stream of the circuit's own) after that
 * run, and returns at once.  The next ps_circuit_run of c waits on the
 * device for the copy to finish reading (it rewrites the same records);
 * runs of other circuits on the same state do not.  Two compiled copies of
 * one circuit on one state, run in turn, so send the records of one run
 * while the next one computes, every run drawing fresh outcomes exactly as
 * consecutive runs of one circuit do.  results / determined (pinned memory
 * for a truly asynchronous copy) must stay valid until ps_circuit_wait_records. */
ps_status ps_circuit_copy_records_async(ps_circuit *c, uint64_t *results, uint64_t *determined, void *copy_stream);
/* Waits for that copy; PS_E_TIMEOUT when the run's sign program gave up on a
 * bounded wait (its records are void). */
ps_status ps_circuit_wait_records(ps_circuit *c);
/* Detectors and observables, computed on the device from the last run's
 * records (no counterpart in the reference, whose callers read records one
 * shot at a time with GetMeasurement): output row d is the XOR of the
 * result rows of the circuit's measurements idx[off[d]] .. idx[off[d+1]-1]
 * (indices in program order, off[0] = 0), for every shot.  out receives
 * ndet rows of `words` uint64 (bit s of word k = shot 64k+s).  Waits for the
 * stream. */
ps_status ps_circuit_detectors(ps_circuit *c, const uint32_t *idx, const uint64_t *off, uint64_t ndet,
                               uint64_t *out);

/* The project's autotuner (no counterpart in the reference): for a circuit
 * with the shared-x/z plan, times its runs over the sign-kernel warps (4, 8)
 * and broadcast CTAs per SM (1, 2); for the per-shot plan (when the
 * circuit's runs take it, or it is built already) times the fused-segment
 * tile shapes (rows x shot-words x threads) on the circuit's first segment
 * and the measurement kernel's shot-words per CTA on its first measurement
 * phase; all on the circuit's own state, keeping the fastest (re-capturing
 * the CUDA graphs).  The tableau and records are left holding
 * valid but meaningless data (runs with reset_state = 1 start over); the
 * event counter is not advanced.  Results are cached per process by
 * (qubits, shot-words, touched qubits), so circuits of one shape are timed
 * once.  *chosen and *tune_ms may be NULL.  Plain circuits are left as they
 * are. */
ps_status ps_circuit_autotune(ps_circuit *c, ps_circuit_options *chosen, double *tune_ms);

/* ------------------------------------------------------ batches of jobs */
/* Many sampling jobs of uneven qubit and shot counts (the reference runs one
 * CliffordState at a time; this has no counterpart there).  Each job is a
 * circuit on its own state, compiled in the fused form; one batch run is ONE
 * CUDA graph launch holding every job as an independent branch, so the
 * device overlaps the jobs' kernels (the small jobs' launches fill the tails
 * of the big ones).  Every job starts from |0...0> and draws from its own
 * seed, exactly as it would alone. */
typedef struct {
    const ps_op *ops;
    uint64_t nops;
    const float *params;
    uint64_t nparams;
    uint64_t num_qubits;
    uint64_t shots;
    int64_t seed;
} ps_job_desc;

typedef struct {
    int32_t autotune;   /* ps_circuit_autotune every job shape first          */
    int32_t use_graph;  /* one graph for the whole batch (else stream order)  */
} ps_batch_options;

typedef struct {
    uint64_t num_jobs;
    uint64_t shot_gates_per_run;  /* sum over jobs of gates x shots          */
    uint64_t tableau_bytes;       /* device bytes of all job tableaux        */
    uint64_t launches_per_run;    /* kernels in one batch run                 */
    double compile_ms, tune_ms;
    uint64_t table_jobs;          /* jobs in the shared-x/z job table: three
                                     launches in all for them                */
    int32_t frame_warps, bcast_ctas; /* the table's knobs (sign-kernel warps
                                        per shot-word, broadcast CTAs per SM) */
} ps_batch_stats;

typedef struct ps_batch ps_batch;
ps_status ps_batch_create(const ps_job_desc *jobs, uint64_t njobs, const ps_batch_options *opts, ps_batch **out);
/* Enqueues one run of every job (returns without waiting). */
ps_status ps_batch_run(ps_batch *b);
ps_status ps_batch_synchronize(ps_batch *b);
/* The stream batch runs are launched on (as void*). */
ps_status ps_batch_get_stream(const ps_batch *b, void **stream);
/* Job j's compiled circuit and state (owned by the batch).  Read records
 * with ps_circuit_copy_records after ps_batch_synchronize. */
ps_status ps_batch_job(const ps_batch *b, uint64_t j, ps_circuit **circuit, ps_state **state);
ps_status ps_batch_get_stats(const ps_batch *b, ps_batch_stats *out);
ps_status ps_batch_destroy(ps_batch *b);

/* ------------------------------------------------------------- serving */
/* A request loop for sampling jobs (no counterpart in the reference).
 * Submitted jobs queue on the host; worker threads admit them while the sum
 * of admitted jobs' device bytes fits the HBM budget and fewer than
 * max_active run, so jobs that arrive while others are on the GPU start as
 * soon as memory and a slot free up, and their kernels overlap on the device
 * (one stream per active job).  The budget is reserved once at creation as
 * one device region; job tableaux, records and scratch come from it and go
 * back to it without device-wide synchronisation.  A job's measurement
 * records are copied to host memory when it finishes and stay there until
 * ps_server_release.  Results are the same as the job run alone: every job
 * starts from |0...0> and draws from its own seed.  A job with no gate that
 * depends on a measurement record holds only its signs, records and noise
 * vectors on the device (no per-shot tableaux: its x / z are the same in
 * every shot and only its records are returned). */
typedef struct {
    uint64_t hbm_budget_bytes;  /* device region for all admitted jobs        */
    int32_t max_active;         /* jobs on the device at once (0 = 16)        */
    int32_t autotune;           /* tune each new job shape on its first job   */
    double hol_wait_s;          /* a queued job that waited this long stops
                                   smaller later jobs from overtaking it      */
    uint64_t host_pool_bytes;   /* pinned host memory for finished jobs'
                                   records (0 = 1 GiB); records that do not
                                   fit go to pageable memory                 */
} ps_server_options;

typedef struct {
    int32_t status;             /* PS_OK, or the job's error code            */
    int32_t pad;
    uint64_t num_measurements;
    uint64_t words;             /* uint64 words per record row                */
    uint64_t shot_gates;
    uint64_t device_bytes;      /* bytes the job held while admitted          */
    double submit_s, admit_s, done_s;  /* server clock (seconds since create) */
    double latency_s;           /* done_s - submit_s                          */
} ps_job_result;

typedef struct {
    uint64_t submitted, completed, failed, queued, active;
    uint64_t cancelled;              /* taken out of the queue by ps_server_cancel */
    uint64_t tableau_jobs;           /* completed jobs that held per-shot tableaux */
    uint64_t shot_gates_completed;
    uint64_t pool_bytes, pool_peak_bytes;
    double p50_latency_s, p99_latency_s, mean_latency_s, max_latency_s;
    double first_submit_s, last_done_s;
} ps_server_stats;

typedef struct ps_server ps_server;
ps_status ps_server_create(const ps_server_options *opts, ps_server **out);
/* Copies the job description and queues it; never blocks on the device.
 * A job larger than the whole budget is refused with PS_E_NOMEM. */
ps_status ps_server_submit(ps_server *s, const ps_job_desc *job, uint64_t *job_id);
/* Park / resume of served jobs (no counterpart in the reference; its import
 * path is HostToDevice, CliffordState.hpp:207-231).  A job submitted with a
 * parked tableau -- x, z ([2n+1][n][words]) and r ([2n+1][words]) packed
 * words of every shot, words = ceil(shots / 64) rounded up to even, as
 * ps_copy_tableau_words gives them -- and event counter starts from them
 * instead of |0...0> and runs its circuit without reset; with keep_tableau
 * its final tableau and event counter are kept for ps_server_copy_tableau.
 * A long job can so leave the device between its parts: each part is a job
 * that resumes the last one's tableau, and the parts' records are those of
 * the whole job run on one state. */
typedef struct {
    const uint64_t *x, *z, *r;  /* parked tableau (all NULL: start from |0...0>) */
    uint64_t events;            /* its event counter                            */
    int32_t keep_tableau;       /* 1: keep the final tableau for ps_server_copy_tableau */
    int32_t pad;
} ps_job_park;
ps_status ps_server_submit_parked(ps_server *s, const ps_job_desc *job, const ps_job_park *park, uint64_t *job_id);
/* The final tableau (the layout above) and event counter of a finished job
 * submitted with keep_tableau (any pointer may be NULL). */
ps_status ps_server_copy_tableau(ps_server *s, uint64_t job_id, uint64_t *x, uint64_t *z, uint64_t *r,
                                 uint64_t *events);
/* Waits up to timeout_s (< 0: no limit) for the job; PS_E_TIMEOUT if it is
 * not done by then. */
ps_status ps_server_wait(ps_server *s, uint64_t job_id, double timeout_s, ps_job_result *out);
/* The finished job's records: num_measurements rows of `words` uint64. */
ps_status ps_server_copy_records(ps_server *s, uint64_t job_id, uint64_t *results, uint64_t *determined);
/* Drops the finished job's host records. */
ps_status ps_server_release(ps_server *s, uint64_t job_id);
/* Takes a job that is still queued out of the queue; waiting for it then
 * reports PS_E_STATE.  A job already admitted runs to its end (its kernels
 * are on the device): PS_E_STATE. */
ps_status ps_server_cancel(ps_server *s, uint64_t job_id);
/* Waits until no job is queued or active (timeout_s < 0: no limit). */
ps_status ps_server_drain(ps_server *s, double timeout_s);
/* Latency percentiles over every job completed so far. */
ps_status ps_server_get_stats(ps_server *s, ps_server_stats *out);
/* Seconds on the server clock. */
ps_status ps_server_now(const ps_server *s, double *seconds);
/* Waits for active jobs, drops queued ones, frees the budget region. */
ps_status ps_server_destroy(ps_server *s);

/* ------------------------------------------------------------ streaming */
/* Block until all work queued on the handle's stream is done. */
ps_status ps_synchronize(ps_state *h);
/* The handle's cudaStream_t (as void*), for callers that order their own work
 * after the library's. */
ps_status ps_get_stream(const ps_state *h, void **stream);
/* Device pointers of the packed tableau planes and their geometry (words per
 * qubit column).  For integration and benchmarking. */
ps_status ps_get_device_tableau(const ps_state *h, void **x, void **z, void **r, uint64_t *words);
/* Copies the packed tableau words [first_word, first_word + nwords) (shots
 * 64*first_word ...) to host memory: x and z as [2n+1][n][nwords], r as
 * [2n+1][nwords] uint64 (any pointer may be NULL).  For checking or
 * snapshotting a shot range of a large state.  Waits for the stream. */
ps_status ps_copy_tableau_words(ps_state *h, uint64_t first_word, uint64_t nwords, uint64_t *x, uint64_t *z,
                                uint64_t *r);
/* The counterpart of ps_copy_tableau_words: loads packed words [first_word,
 * first_word + nwords) of x, z ([2n+1][n][nwords]) and r ([2n+1][nwords])
 * from host memory (any pointer may be NULL: that plane is kept).  With the
 * event counter (ps_set_event_counter) it resumes a state snapshotted by
 * ps_copy_tableau_words, shot range by shot range: the import path of
 * HostToDevice (CliffordState.hpp:207-231) in the packed layout, without
 * the int32 expansion.  Waits for the copy. */
ps_status ps_load_tableau_words(ps_state *h, uint64_t first_word, uint64_t nwords, const uint64_t *x,
                                const uint64_t *z, const uint64_t *r);
/* DeviceToDevice (CliffordState.hpp:268-274): copies packed device planes of
 * the same geometry (another state's ps_get_device_tableau, whose work must
 * be finished) into h's tableau.  Waits for the copy. */
ps_status ps_device_to_device(ps_state *h, const void *x, const void *z, const void *r);
/* Device pointers of record `id` (packed words, ps_get_device_tableau's
 * word count): the counterpart of Measurement::measurement_results_device /
 * measurement_determined_device (CliffordState.hpp:36-37). */
ps_status ps_get_record_device(ps_state *h, uint64_t id, void **results, void **determined);

#ifdef __cplusplus
}
#endif
#endif /* PLAQUETTE_GPU_H */
