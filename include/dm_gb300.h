/*
 * dm_gb300.h -- C ABI of the GB300 Pauli-basis density-matrix engine.
 *
 * The state of an n-qubit register is the real vector a[4**n] of Pauli
 * coefficients, rho = sum_s a_s sigma_{s_0} x ... x sigma_{s_{n-1}}, with
 * flat index s = sum_q p_q * 4**(n-1-q), p in {0:I, 1:X, 2:Y, 3:Z}
 * (qubit 0 is the slowest axis), exactly the layout of the reference's
 * ``DmSimulatorPy._densitymatrix`` (qiskit/providers/basicaer/dm_simulator.py
 * :62-67, :376).  It lives in GPU memory as FP64 (DM_F64) or FP32 (DM_F32).
 *
 * Conventions
 *   - Every entry point returns 0 on success or a negative DM_ERR_* code; no
 *     C++ exception crosses this boundary.  dm_error_string() names a code.
 *   - Pointers named *_dev are device pointers; everything else is host.
 *   - ``stream`` is a cudaStream_t passed as void* (NULL = legacy stream).
 *     Work is enqueued asynchronously; host outputs are written before return.
 *   - Small matrices (4x4, 16x16, row-major, output row x input column) are
 *     passed by host pointer and copied into the kernel's parameters.
 *   - No entry point allocates device memory; callers pass scratch buffers
 *     sized by the matching *_scratch_bytes() query.
 *
 * Each entry point names the reference function it replaces.
 */
#ifndef DM_GB300_H
#define DM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum dm_dtype { DM_F64 = 0, DM_F32 = 1 };

enum dm_status {
    DM_OK = 0,
    DM_ERR_ARG = -1,      /* invalid argument (qubit index, size, dtype, pointer) */
    DM_ERR_CUDA = -2,     /* a CUDA runtime call failed (launch, copy) */
    DM_ERR_RANGE = -3,    /* size beyond a documented limit */
    DM_ERR_PROGRAM = -4   /* malformed fused-pass program */
};

/* Limits of the fused-pass kernel. */
#define DM_MAX_QUBITS 17            /* 4**17 FP64 = 137 GB: the largest state one GB300 holds */
#define DM_MAX_TILE_AXES 7          /* resident axes of one tile (4**7 coefficients) */
#define DM_MAX_PASS_OPS 128         /* operations applied to one tile in one pass */
#define DM_MAX_ROUNDS 48            /* register rounds of one pass */

/* Operation kinds of a fused pass (local axes index the pass's resident axes). */
enum dm_op_kind {
    DM_OP_MAP1 = 1,    /* 4x4 real map on local axis a; mat = 16 entries */
    DM_OP_MAP2 = 2,    /* 16x16 real map on local axes (a, b), index 4*p_a + p_b; mat = 256 entries */
    DM_OP_DIAG2 = 3,   /* diagonal of a 16x16 map on (a, b); mat = 16 entries */
    DM_OP_CX = 4       /* CX with control on local axis a, target on b; mat = 5 coefficients
                          (c, s, c2, s2, cs) of basicaertools.py:329-336 */
};

/* flags of DM_OP_MAP1 */
#define DM_MAP1_ROW0_IDENTITY 1   /* row 0 of the map is (1,0,0,0): the I component is unchanged */
#define DM_MAP1_XY_UNITAL 2       /* entries (1,0) and (2,0) are 0: X and Y take no I component
                                     (register rounds only; with ROW0_IDENTITY: 10 FMAs per 4 values) */
/* flags of DM_OP_CX */
#define DM_CX_IDEAL 1             /* (c,s,c2,s2,cs) = (1,0,1,0,0): a signed permutation */

typedef struct dm_op {
    int32_t kind;
    int16_t a, b;
    int32_t flags;
    int32_t moff;       /* offset of the op's coefficients in the pass's matrix buffer */
} dm_op;

typedef struct dm_pass {
    int32_t k;                          /* number of resident axes, 1..DM_MAX_TILE_AXES */
    int32_t axes[DM_MAX_TILE_AXES];     /* qubit of local axis r; strictly decreasing (local axis 0
                                           has the smallest stride) */
    int32_t nops;
    /* Register rounds.  nrounds = 0: the ops are applied one at a time to the
     * shared-memory tile.  nrounds > 0: the ops are grouped into rounds; in
     * round r every thread holds groups of 4**R coefficients spanning the
     * round's R local axes round_axes[r][0..R-1] (ascending; R = 3 for FP32,
     * 2 for FP64) in registers and applies ops [round_end[r-1], round_end[r])
     * (each acting only on the round's axes) before writing them back. */
    int32_t nrounds;
    int8_t round_axes[DM_MAX_ROUNDS][4];
    int16_t round_end[DM_MAX_ROUNDS];
    dm_op ops[DM_MAX_PASS_OPS];
} dm_pass;

/* Round width (axes held in registers per round) for a dtype. */
#define DM_ROUND_AXES_F32 3
#define DM_ROUND_AXES_F64 2

/* ---------------------------------------------------------------- state set-up */

/* Product state a[s] = scale * prod_q v[q][s_q] (v: n x 4, host).
 * Replaces DmSimulatorPy._initialize_densitymatrix, dm_simulator.py:284-349
 * (all-zero, max_mixed, uniform_superpos, thermal_state and binary_string
 * states are Kronecker products of per-qubit 4-vectors scaled by 2**-n). */
int dm_init_product(void *state_dev, int n, int dtype, const double *v, double scale, void *stream);

/* Copy a host FP64 coefficient vector (4**n) into the state (converting to dtype).
 * Replaces the stored_density_matrix path, dm_simulator.py:337-343. */
int dm_load_state(void *state_dev, int n, int dtype, const double *host_coeffs, void *stream);

/* ------------------------------------------------------------ gates and noise */

/* One 4x4 map on the Pauli axis of qubit q.
 * Replaces rot_gate_dm_matrix (basicaertools.py:93-126) as used by
 * DmSimulatorPy._add_unitary_single (dm_simulator.py:367-384), the per-qubit
 * measurement updates (dm_simulator.py:574-704) and reset (:810-823). */
int dm_apply_map1(void *state_dev, int n, int dtype, int q, const double *m4x4, void *stream);

/* CX with control qc and target qt under the transition-selective-pulse error
 * model err = (<cos a>, mean a).  Replaces cx_gate_dm_matrix,
 * basicaertools.py:310-392 (via DmSimulatorPy._add_unitary_two, dm_simulator.py:386-395). */
int dm_apply_cx(void *state_dev, int n, int dtype, int qc, int qt, const double *tsp_err2, void *stream);

/* Memory noise on every qubit: X,Y *= sqrt(g)*f ; Z <- g*Z + (1-g)(2p-1)*I.
 * Replaces DmSimulatorPy._add_decoherence_and_amp_decay, dm_simulator.py:397-425. */
int dm_apply_memory_noise(void *state_dev, int n, int dtype, double f, double p, double g, void *stream);

/* A fused pass: every tile of 4**k coefficients spanned by the pass's
 * resident axes is loaded once, all of the pass's operations are applied to
 * it on chip, and it is written back once.  mats_dev holds mats_count
 * coefficients (in the state's dtype) that the ops index by moff.  This is the GB300 form of a run of
 * consecutive levels of DmSimulatorPy.run_experiment (dm_simulator.py:1005-1177).
 * With nrounds > 0 the pass runs on the pipelined round kernel, which needs
 * the lowest qubit axis (n-1) resident, at most 7 (FP32) / 6 (FP64)
 * resident axes, no DM_OP_MAP2, and a 16-byte aligned state. */
int dm_apply_pass(void *state_dev, int n, int dtype, const dm_pass *pass, const void *mats_dev,
                  size_t mats_count, void *stream);

/* A tensor-core pass.  Every tile of 4**7 coefficients (the 7 resident
 * axes) is viewed, round by round, as a 256 x 64 FP16 operand: rows are
 * groups, K the 64 coefficients of the round's 3 axes, stored in the K-major
 * core-matrix layout byte(row, k) = (row%8)*16 + (k%8)*2 + (k/8)*128 +
 * (row/8)*1024.  A round is D = X U^T with U the 64x64 transfer matrix of
 * its composed operations.  Layout offsets are XOR-combinations of one
 * offset per index bit (every operand-layout bit contributes a distinct
 * power of two, and the natural tile layout is XOR-linear). */
typedef struct dm_tc_round {
    int8_t digits[3];     /* local axes of K digits 0, 1, 2 (j = d0 + 4 d1 + 16 d2) */
    int8_t vec;           /* digit whose 4 values the epilogue stores as one vector (8 bytes of FP16 into
                             the next operand, 16 bytes of FP32 into the natural tile), or -1 */
    int32_t umoff;        /* FP16-value offset of the round's matrix images: 2**11 Uh, Ul, Uh (4096 each),
                             value (n%8)*8 + k%8 + (k/8)*64 + (n/8)*512 for output n, input k */
    uint32_t rowc[8];     /* destination offset of row bit i of this round: bytes into the next round's
                             operand, or, after the last round, elements of the natural tile */
    uint32_t kc[6];       /* destination offset of K bit i of this round */
} dm_tc_round;

typedef struct dm_tc_pass {
    int32_t axes[7];      /* resident qubits, strictly decreasing; axes[0] must be n-1 */
    int32_t nrounds;
    int8_t vec0;          /* 0 when round 0's digit 0 is local axis 0 (128-bit conversion loads), else -1 */
    int8_t direct_last;   /* dm_apply_pass_tc and the batched tensor-core sweeps: 1 = the last round stores
                             straight to global memory (its rowc / kc are the linear natural offsets 2**b
                             of tile bits b, rows 0-3 on tile bits 0-3) and the next tile's load overlaps
                             it; 0 = through the natural tile in shared memory.  dm_apply_pass_tma always
                             stores its last round directly and ignores this field. */
    int8_t pad[2];
    uint32_t natrow[8];   /* natural-tile element offset of round 0's row bit i */
    uint32_t natk[6];     /* natural-tile element offset of round 0's K bit i */
    dm_tc_round rounds[DM_MAX_ROUNDS];
} dm_tc_pass;

/* The fused pass on the tensor cores (FP32 state only, n >= 7): the rounds
 * run as tcgen05.mma kind::f16 on a 3-way FP16 split (the tile in units of
 * 2**-n, x = h + 2**-11 l; U = Uh + 2**-11 Ul; FP32 accumulators in
 * tensor memory collect h (2**11 Uh)^T and h Ul^T + l Uh^T).  The state must
 * be physical enough that |2**n a| < 65504.  umats_dev holds umats_count
 * FP16 values (uint16_t bits).  status_dev (device int, 0 before the first
 * call) is set to 1 if the kernel abandons a bounded wait.  Same role as
 * dm_apply_pass (dm_simulator.py:1005-1177). */
int dm_apply_pass_tc(void *state_dev, int n, const dm_tc_pass *pass, const uint16_t *umats_dev, size_t umats_count,
                     int *status_dev, void *stream);

/* The same pass with TMA-fed tiles: one CTA per SM of two thread teams,
 * each streaming its tiles through its own shared-memory slot by
 * cp.async.bulk.tensor loads and stores, with the pass's round images
 * resident in shared memory.  Differences from dm_apply_pass_tc: the
 * natural-tile tables (natrow / natk, and rowc / kc of the last round) are
 * plain element offsets (the TMA box is unswizzled); each round's images are
 * 8192 FP16 values, Uh then Ul = fp16(2**11 (U - Uh)) (no 2**11 Uh image);
 * at most 16 rounds (up to 6 with every image resident in shared memory,
 * the later ones streamed per round); the resident axes must fit a 5-dimensional tensor map
 * (runs of consecutive qubits, at most 4 per dimension).  Returns
 * DM_ERR_PROGRAM for a pass outside these limits (the caller then uses
 * dm_apply_pass_tc).  Same role as dm_apply_pass (dm_simulator.py:1005-1177). */
int dm_apply_pass_tma(void *state_dev, int n, const dm_tc_pass *pass, const uint16_t *umats_dev, size_t umats_count,
                      int *status_dev, void *stream);

/* out_dev[0] = max |a_s - b_s| over the 4**n coefficients of two device states
 * (dtypes DM_F32 / DM_F64 each), computed in FP64 on the device.  The error
 * statement of an FP32 result against the same experiment run in FP64
 * (no reference counterpart: the reference computes in FP64 only). */
int dm_max_abs_diff(const void *a_dev, int dtype_a, const void *b_dev, int dtype_b, int n, double *out_dev,
                    void *stream);

/* FP64 FMA throughput probe (measurement only, no reference counterpart):
 * dm_fp64_fma_probe_threads() threads each run 8 independent chains of
 * `iters` FMAs and write one double each into out_dev (that many doubles).
 * FP64 FLOPs of one launch: 2 * 8 * iters * threads.  bench.py times it to
 * state the FP64 pipe's measured peak beside the FP64 pass's throughput. */
int dm_fp64_fma_probe_threads(void);
int dm_fp64_fma_probe(double *out_dev, int64_t iters, void *stream);

/* Tile-pattern copy probe (measurement only, no reference counterpart):
 * reads and writes the FP32 state at state_dev (4**n values) in place, tile by
 * tile, for the 7 resident qubits axes[0..6] (strictly decreasing, axes[0] =
 * n-1) with 16-byte accesses and no change to any value.  Its rate is the DRAM
 * rate this tile shape allows; bench.py times it over the tiles of the
 * headline's tensor-core passes beside their own rate. */
int dm_tile_copy_probe(float *state_dev, int n, const int32_t *axes, void *stream);

/* Page-locked host memory mapped into the device's address space
 * (cudaHostAlloc, mapped and portable), exactly `bytes` long, or NULL.  The
 * copy-out writes a result block of this kind directly from the chop kernel
 * (dm_chop_copy with out_dev = dm_host_device_pointer(block)), in one pass
 * over the CPU-GPU link, with no device staging buffer.  No reference
 * counterpart (the reference's state lives in host memory). */
void *dm_host_alloc(size_t bytes);
void *dm_host_device_pointer(void *host);
int dm_host_free(void *host);

/* Self-test of the tensor-core kernels' bounded waits (no reference
 * counterpart): one thread waits on an mbarrier that nothing arrives on, gives
 * up after limit_ns (0 < limit_ns <= 1e8) and sets *status_dev = 1, the status
 * a pass kernel reports when a wait for an MMA commit or a tile load runs out.
 * Lets a test check the failure path without faulting or hanging a GPU. */
int dm_tc_wait_selftest(int *status_dev, int64_t limit_ns, void *stream);

/* ------------------------------------------------------------------ levelling */

/* Instruction kinds for dm_levelize. */
#define DM_SCHED_GATE1 1      /* u1 / u3 on one qubit (after the single-gate merge) */
#define DM_SCHED_CX 2
#define DM_SCHED_MEASURE 3
#define DM_SCHED_RESET 4
#define DM_SCHED_BARRIER 5
#define DM_SCHED_OTHER 6      /* anything else: cannot be placed (DM_ERR_PROGRAM) */

/* Levels (clock cycles) of a merged instruction list, host code: replaces
 * partition / partition_helper / qubit_stack, basicaertools.py:536-749.
 * Instruction i has kind[i] and qubits qubits[qoff[i] .. qoff[i+1]-1]
 * (qoff has count + 1 entries, qoff[0] = 0).  Every instruction other than
 * a barrier is placed once: placed_inst[k] (instruction index) goes to entry
 * placed_pos[k] of the level table, in placement order (the order the
 * reference appends them); *placed_count placements.  *table_len is the
 * length of the concatenated per-piece tables (unused trailing entries
 * included) and *levels the number of executed levels (the reference's
 * number_of_clock_cycles): the first *levels entries run.  placed_inst and
 * placed_pos hold count entries each.  DM_ERR_PROGRAM when an instruction can
 * never be placed. */
int dm_levelize(int n, int count, const int32_t *kind, const int32_t *qoff, const int32_t *qubits,
                int32_t *placed_inst, int32_t *placed_pos, int32_t *placed_count, int32_t *table_len,
                int32_t *levels);

/* ------------------------------------------------------------- batched sweeps */

/* One pass of a batched program (the n-independent part of dm_pass). */
typedef struct dm_batch_pass {
    int8_t k;                          /* resident axes; axes[0] must be the instance's qubit n-1 */
    int8_t nrounds;
    int16_t nops;
    int8_t axes[DM_MAX_TILE_AXES];     /* resident qubits, strictly decreasing */
    int8_t pad;
    int8_t round_axes[DM_MAX_ROUNDS][4];
    int16_t round_end[DM_MAX_ROUNDS];
    dm_op ops[DM_MAX_PASS_OPS];        /* moff relative to the instance's coefficient block */
} dm_batch_pass;

/* Round image formats of dm_compose_rounds. */
#define DM_IMAGE_TC 1    /* 12288 FP16 values per round: 2**11 Uh | Ul | Uh (dm_apply_pass_tc) */
#define DM_IMAGE_TMA 2   /* 8192 FP16 values per round: Uh | Ul (dm_apply_pass_tma) */

/* The round images of one tensor-core pass, composed in FP64 on the device:
 * round r's 64x64 transfer matrix U (input and output index j = d0 + 4 d1
 * + 16 d2 over the round's local axes pass->round_axes[r][0..2]) is ops
 * [round_end[r-1], round_end[r]) applied to the 64 unit vectors, written at
 * images_dev + r * (values per round) as Uh = fp16(U) and
 * Ul = fp16(2**11 (U - Uh)) in the K-major core-matrix order the passes
 * read.  Op coefficients (moff in doubles) come from mats_dev; ops may be
 * DM_OP_MAP1, DM_OP_MAP2, DM_OP_DIAG2 and DM_OP_CX, with their digit
 * positions in the flags as in the register rounds.  pass->k and
 * pass->axes are not read.  One launch of nrounds CTAs, stream-ordered
 * before the pass that reads the images.  The reference multiplies the
 * same per-gate maps one gate at a time on the host (dm_simulator.py:1005-1177);
 * here they are folded into one matrix per round. */
int dm_compose_rounds(int format, const dm_batch_pass *pass, const double *mats_dev, size_t mats_count,
                      uint16_t *images_dev, size_t images_count, void *stream);

/* One independent circuit instance of a batched program. */
typedef struct dm_batch_instance {
    int32_t n;                         /* qubits */
    int32_t npasses;                   /* passes pass_begin .. pass_begin + npasses - 1 */
    int32_t pass_begin;
    int32_t pad;
    int64_t state_off;                 /* element offset of the instance's 4**n state */
    int64_t prob_off;                  /* double offset of its 2**n outcome probabilities */
    int64_t mats_off;                  /* element offset of its coefficient block */
    int64_t mats_len;                  /* elements in its coefficient block */
    double meas_err;                   /* polarisation of the final Z measurement of every qubit */
} dm_batch_instance;

/* Run many independent circuit instances in one persistent launch: every
 * CTA takes the next instance from a work counter (the caller orders the
 * instances largest first), prepares |0...0>, applies the instance's passes
 * with the pipelined register-round kernel and writes the 2**n probabilities
 * of a Z measurement of every qubit (polarisation meas_err), the read-out of
 * DmSimulatorPy._add_ensemble_measure (dm_simulator.py:427-481).
 * The tables are passed twice: host copies (validated here) and the
 * identical device copies the kernel reads.  counter_dev is reset here
 * (cudaMemsetAsync), so the call can be captured in a CUDA graph after a
 * first call.  status_dev is left 0.  dtype F32 (3-axis rounds, passes of
 * <= 7 axes) or F64 (2-axis rounds, <= 6 axes). */
int dm_batch_run(int dtype, void *states_dev, size_t states_count, double *probs_dev, size_t probs_count,
                 const void *mats_dev, size_t mats_count, const dm_batch_instance *insts_host,
                 const dm_batch_instance *insts_dev, int ninst, const dm_batch_pass *passes_host,
                 const dm_batch_pass *passes_dev, int npasses, int *counter_dev, int *status_dev, void *stream);

/* One pass of a batched program on the tensor cores: 7 resident axes, every
 * round a 64x64 transfer matrix composed on the device from the instance's
 * own coefficients.  ops.k = 7; ops.round_axes[r][0..2] are round r's local
 * axes in K-digit order (they must equal tables.rounds[r].digits) and the
 * digit positions in the op flags refer to that order; tables holds the
 * conversion and epilogue tables (tables.axes and rounds[].umoff are not
 * read). */
typedef struct dm_batch_tc_pass {
    dm_batch_pass ops;
    dm_tc_pass tables;
} dm_batch_tc_pass;

/* Device scratch dm_batch_run_tc needs for the round matrices it composes
 * (DM_MAX_ROUNDS FP16 image sets per CTA). */
size_t dm_batch_tc_scratch_bytes(void);

/* dm_batch_run for FP32 instances of 7..12 qubits with every pass on the
 * tensor cores (the dm_apply_pass_tc kernel): at the start of each pass a
 * CTA composes the pass's round matrices from the instance's FP64
 * coefficient block (the ops applied to the 64 unit vectors, in FP64) into
 * its slice of scratch_dev as the 3-way FP16 split images, then streams the
 * instance's tiles.  status_dev is set to 1 if a bounded tensor-core wait
 * gives up. */
int dm_batch_run_tc(float *states_dev, size_t states_count, double *probs_dev, size_t probs_count,
                    const double *mats_dev, size_t mats_count, const dm_batch_instance *insts_host,
                    const dm_batch_instance *insts_dev, int ninst, const dm_batch_tc_pass *passes_host,
                    const dm_batch_tc_pass *passes_dev, int npasses, int *counter_dev, void *scratch_dev,
                    size_t scratch_bytes, int *status_dev, void *stream);

/* Parametric batched programs: every instance runs the same circuit
 * template (one plan) and differs only in its noise parameters.  Each
 * operation of the template is a recipe; a slot of a pass composes a chain
 * of recipes (application order) in FP64 on the GPU, per instance and per
 * pass, from the instance's parameter vector:
 *   params[0..2]  decoherence f, thermal p, decay g   (memory noise, dm_simulator.py:397-425)
 *   params[3..8]  rotation error (<cos>, mean) of rx, ry, rz   (basicaertools.py:93-126)
 *   params[9..10] CX transition model error (<cos>, mean)      (basicaertools.py:329-336)
 *   params[11]    measurement polarisation of the final Z read-out */
#define DM_PARAMS_MIN_STRIDE 12
#define DM_RECIPE_ROT 1     /* up to 3 rotations (axis 0 rx, 1 ry, 2 rz) by fixed angles, instance errors */
#define DM_RECIPE_NOISE 2   /* memory noise of the instance's f, p, g */
#define DM_RECIPE_CX 3      /* CX coefficients of the instance's transition model error */
#define DM_RECIPE_CONST 4   /* a fixed 4x4 map (or 16-entry diagonal pair map): 16 values in consts */

typedef struct dm_recipe {
    int8_t kind;
    int8_t nrot;
    int8_t axis[3];
    int8_t pad[3];
    int32_t const_off;
    int32_t pad2;
    double angle[3];
} dm_recipe;

typedef struct dm_param_slot {
    int32_t begin, len;                /* recipe indices chain[begin .. begin + len - 1] */
} dm_param_slot;

/* One template program.  The passes are dm_batch_pass tables (op moff is
 * ignored: a pass's coefficients are composed into shared memory); slot s
 * of the program is op s of the concatenated passes. */
typedef struct dm_param_program {
    int32_t n, npasses, nslots, nchain, nrecipes, nconsts;
    const dm_batch_pass *passes;
    const dm_param_slot *slots;
    const int32_t *chain;
    const dm_recipe *recipes;
    const double *consts;
} dm_param_program;

/* Run ninst instances of one template in one persistent launch: instance i
 * starts in |0...0>, runs the passes with its own parameters
 * (params_dev + i * params_stride) and writes the 2**n probabilities of a
 * Z measurement of every qubit to probs_dev + i * 2**n; its state lives at
 * states_dev + i * 4**n.  host holds host copies of the tables (validated
 * here), dev the identical device copies the kernel reads.  The call resets
 * counter_dev and can be captured in a CUDA graph after a first call. */
int dm_batch_run_params(int dtype, const dm_param_program *host, const dm_param_program *dev,
                        const double *params_dev, int params_stride, int ninst, void *states_dev,
                        size_t states_count, double *probs_dev, size_t probs_count, int *counter_dev, void *stream);

/* dm_batch_run_params with every pass on the tensor cores (FP32, 7 <= n <=
 * 12): the passes are tensor-core passes (passes_host / passes_dev, npasses
 * = host->npasses; host->passes is not read), op o of each pass with moff =
 * 16 o.  Per instance and pass the slots' recipe chains are composed in FP64,
 * then the round matrices from them (as in dm_batch_run_tc) into scratch_dev
 * (dm_batch_tc_scratch_bytes), then the tiles run.  status_dev is set to 1
 * if a bounded tensor-core wait gives up. */
int dm_batch_run_params_tc(const dm_param_program *host, const dm_param_program *dev,
                           const dm_batch_tc_pass *passes_host, const dm_batch_tc_pass *passes_dev,
                           const double *params_dev, int params_stride, int ninst, float *states_dev,
                           size_t states_count, double *probs_dev, size_t probs_count, int *counter_dev,
                           void *scratch_dev, size_t scratch_bytes, int *status_dev, void *stream);

/* ---------------------------------------------------------- noise surrogate
 *
 * No counterpart in the reference.  A small MLP ensemble learns the map from
 * noise parameters to a fixed circuit's Z outcome distribution from data
 * that the batched sweep generates; the plain simulation stays the fallback
 * wherever the ensemble disagrees with itself.  These entry points are the
 * network's kernels: a tcgen05 BF16 GEMM with fused epilogues, softmax with
 * the KL loss and its gradient, bias gradients, Adam, the minibatch gather
 * and the ensemble statistics.  BF16 values travel as uint16_t bit patterns.
 * Every call works on `members` independent networks at once (member i adds
 * i times the *_ms stride, in elements, to each of its pointers). */

#define DM_MLP_EPI_GELU_FWD 0   /* u = acc + bias: out_f32 = u (optional), out_bf16 / out_t = gelu(u) */
#define DM_MLP_EPI_BIAS_F32 1   /* out_f32 = acc + bias */
#define DM_MLP_EPI_GELU_BWD 2   /* d = acc * gelu'(pre): out_bf16 / out_t = d */
#define DM_MLP_EPI_F32 3        /* out_f32 = acc */

/* C[M x N] = A[M x K] * B[N x K]^T, BF16 operands (row-major, K contiguous),
 * FP32 accumulation in tensor memory, then the epilogue.  M % 128 == 0,
 * N % 64 == 0, K % 64 == 0; leading dimensions and member strides are
 * multiples of 8 elements and every pointer is 16-byte aligned.  out_t is
 * the transposed [N x M] copy (optional). */
typedef struct dm_mlp_gemm {
    int32_t epi, M, N, K, members, pad;
    const uint16_t *A;
    int64_t lda, a_ms;
    const uint16_t *B;
    int64_t ldb, b_ms;
    const float *bias;
    int64_t bias_ms;
    const float *pre;
    int64_t ld_pre, pre_ms;
    float *out_f32;
    int64_t ld_f32, f32_ms;
    uint16_t *out_bf16;
    int64_t ld_bf16, bf16_ms;
    uint16_t *out_t;
    int64_t ld_t, t_ms;
} dm_mlp_gemm;

/* status_dev is set to 1 if a bounded wait for the tensor cores gave up. */
int dm_mlp_gemm_run(const dm_mlp_gemm *g, int *status_dev, void *stream);

/* Row softmax of logits [members][rows][nout]; with targets (same shape),
 * loss_rows[members][rows] = KL(t || q) per row and the gradient
 * d = (q - t) * grad_scale as BF16 dz [members][rows][nout] and its
 * transpose dzt [members][nout][rows].  probs (optional) receives q.
 * nout % 256 == 0, nout <= 4096. */
int dm_mlp_softmax_xent(const float *logits, const float *targets, int rows, int members, int nout,
                        float grad_scale, float *probs, uint16_t *dz, uint16_t *dzt, float *loss_rows, void *stream);

/* db[n] = sum over b < rows of d_t[n * ld + b] (BF16 in, FP32 out), n < N. */
int dm_mlp_bias_grad(const uint16_t *d_t, int64_t ld, int64_t d_ms, int N, int rows, int members, float *db,
                     int64_t db_ms, void *stream);

/* One Adam step over every parameter of `members` networks laid out as
 * W1 b1 W2 b2 ... (W row-major [out x in]); shapes holds (out, in) per layer
 * (host array, nlayers <= 8).  step <= 0 only refreshes the BF16 copies:
 * w_bf16 (same layout) and wt_bf16 (each W transposed [in x out] at the
 * same offset). */
int dm_mlp_adam(float *params, const float *grads, float *m, float *v, int64_t count_per_member, int members,
                const int32_t *shapes, int nlayers, float lr, float beta1, float beta2, float eps, int step,
                uint16_t *w_bf16, uint16_t *wt_bf16, void *stream);

/* Minibatch gather: for member z and row r, sample s = index[z * rows + r]:
 * x[z][r][f] and xt[z][f][r] = features[s][f] (BF16, zero for
 * nfeat <= f < width) and, unless targets is NULL, t[z][r][:] = targets[s][:]
 * (nout FP32 values).  An index outside [0, samples) reads sample 0.
 * width % 8 == 0, nout % 4 == 0. */
int dm_mlp_gather(const float *features, int nfeat, const float *targets, int nout, int64_t samples,
                  const int32_t *index, int rows, int members, int width, uint16_t *x, uint16_t *xt, float *t,
                  void *stream);

/* Ensemble statistics of probs [members][rows][nout]: mean [rows][nout],
 * spread[r] = mean over members of TV(q_member, mean) and, with ref
 * [rows][nout], tv_ref[r] = TV(mean, ref).  members <= 8. */
int dm_mlp_ensemble(const float *probs, int rows, int members, int nout, const float *ref, float *mean,
                    float *spread, float *tv_ref, void *stream);

/* ---------------------------------------------------------------- measurement */

/* Probabilities of a measurement along one Pauli axis per qubit.
 * mode[q] = 0: qubit q is not measured (marginalised);
 *           1..3: measured along X, Y or Z with polarisation err.
 * Outputs 2**m probabilities (m = number of measured qubits, the lowest
 * measured qubit is the most significant bit) into out_dev (FP64, 2**m).
 * With every qubit measured this replaces DmSimulatorPy._add_ensemble_measure
 * (dm_simulator.py:427-481) for bases X/Y/Z; with some qubits unmeasured it
 * gives the probabilities of _add_partial_measure (dm_simulator.py:492-538):
 * only the 2**m coefficients on the measured sub-lattice are read, and a
 * Walsh-Hadamard transform in out_dev turns them into probabilities. */
int dm_axis_probs(const void *state_dev, int n, int dtype, const int *mode, double err,
                  double *out_dev, void *stream);

/* Probabilities of an ensemble measurement along the direction nvec (basis N,
 * dm_simulator.py:456-462), every qubit measured: 2**n FP64 outputs.
 * scratch_dev: dm_nbasis_probs_scratch_bytes(n) bytes. */
size_t dm_nbasis_probs_scratch_bytes(int n);
int dm_nbasis_probs(const void *state_dev, int n, int dtype, const double *nvec3, double err,
                    double *out_dev, void *scratch_dev, void *stream);

/* dm_nbasis_probs for callers that cannot allocate device memory.
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc -- code whose device memory is already handed to another
 * allocator (a framework's caching pool) where raw allocations fail or are
 * not allowed, and code on a latency-critical path where cudaMalloc/cudaFree
 * would synchronise the device.  The caller still passes the state and the
 * 2**n output; the scratch is a file-scope device array of 196,608 doubles
 * (1.5 MiB), which every GPU that loads this library holds until the process
 * exits, enough for n <= 10.  Larger n returns DM_ERR_RANGE without touching
 * the GPU.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current), so make that first call
 * before any stream capture; the address is looked up again when the
 * device's CUDA context has changed since (after cudaDeviceReset the module,
 * and with it the array, may sit elsewhere).  Every call shares the one array: calls that
 * overlap on the GPU (other streams, other host threads) race on it.  Each
 * call writes every scratch element it reads, so nothing left from a previous
 * call reaches a result.  Allocates nothing (no cudaMalloc / cudaFree). */
int dm_nbasis_probs_noalloc(const void *state_dev, int n, int dtype, const double *nvec3, double err,
                            double *out_dev, void *stream);

/* Gather count coefficients a[idx[i]] (FP64) into out_dev.  Used for the
 * Pauli-string expectation (dm_simulator.py:569-570), the Bell reduced matrix
 * and probabilities (:744-760) and the trace check (:363). count <= 64. */
int dm_gather(const void *state_dev, int n, int dtype, const int64_t *idx, int count,
              double *out_dev, void *stream);

/* Shot counts from 2**m outcome probabilities (FP64, device), no counterpart
 * in the reference (its dm_simulator has max_shots = 1 and reports
 * probabilities only).  counts_dev receives 2**m int64 counts summing to
 * shots; the draws are a deterministic function of seed.  Negative
 * probabilities count as 0; when none is positive, no shot is drawn and
 * every count is 0 (so the counts sum to 0, not shots).  m <= 20;
 * scratch_dev: dm_sample_counts_scratch_bytes(m) bytes. */
size_t dm_sample_counts_scratch_bytes(int m);
int dm_sample_counts(const double *probs_dev, int m, int64_t shots, uint64_t seed, int64_t *counts_dev,
                     void *scratch_dev, void *stream);

/* ------------------------------------------------------------------ outputs */

/* out[s] = a[s], with |a[s]| < threshold set to 0 (FP64 output, 4**n).
 * Replaces DmSimulatorPy._get_densitymatrix's chop, dm_simulator.py:1257-1269. */
int dm_chop_copy(const void *state_dev, int n, int dtype, double threshold, double *out_dev, void *stream);

/* dm_chop_copy of coefficients offset .. offset + count - 1 only (out_dev holds count
 * values), so a large state can be copied out in chunks that overlap the host copies. */
int dm_chop_copy_range(const void *state_dev, int n, int dtype, int64_t offset, int64_t count, double threshold,
                       double *out_dev, void *stream);

/* Pauli basis -> 2**n x 2**n complex128 matrix (interleaved re/im, row-major).
 * Replaces DmSimulatorPy._compute_densitymatrix, dm_simulator.py:1198-1255.
 * scratch_dev: dm_pauli_to_matrix_scratch_bytes(n) bytes. */
size_t dm_pauli_to_matrix_scratch_bytes(int n);
int dm_pauli_to_matrix(const void *state_dev, int n, int dtype, double *out_dev, void *scratch_dev,
                       void *stream);

/* out_dev[0] = 2**n * sum_s a[s] b[s] (FP64).  Replaces DmSimulatorPy._state_overlap,
 * dm_simulator.py:1277-1282.  scratch_dev: dm_overlap_scratch_bytes(n) bytes. */
size_t dm_overlap_scratch_bytes(int n);
int dm_overlap(const void *a_dev, const void *b_dev, int n, int dtype, double *out_dev,
               void *scratch_dev, void *stream);

/* ---------------------------------------------------------------------- misc */

const char *dm_error_string(int code);
/* Number of kernels this library has launched since load (all entry points). */
uint64_t dm_kernel_launch_count(void);
/* Library version, e.g. "dm_gb300 1.0 sm_103a". */
const char *dm_version(void);

#ifdef __cplusplus
}
#endif
#endif /* DM_GB300_H */
