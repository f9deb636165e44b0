/*
 * spinwalk_gpu.h -- C ABI of libspinwalk_gpu.so, the GB300 (sm_103a) implementation of
 * SpinWalk's `sim` hot path: the per-spin Monte-Carlo random walk over a voxel phantom with
 * the Bloch update.
 *
 * Every entry point returns an int status (SW_OK or a negative SW_ERR_* code) and never exits
 * or traps; sw_last_error() gives a one-line message for the last failure on the calling thread.
 * No torch or CUDA types appear in the signatures: streams are passed as `void*`
 * (a cudaStream_t, NULL = legacy default stream).
 *
 * Reference interfaces replaced (paths relative to the SpinWalk 1.21.0 source tree):
 *   sw_params            <- struct sim::parameters          src/sim/simulation_parameters.cuh:176-246
 *   sw_sequence          <- struct parameters_uvec          src/sim/simulation_parameters.cuh:102-173
 *   sw_sim               <- std::for_each(par_unseq, sim::sim) over all spins of one scale
 *                           src/sim/monte_carlo.cu:313-321 (host buffers in, host buffers out)
 *   sw_sim_device        <- cu_sim<<<ceil(n/256),256>>>(...) + gpuCheckKernelExecutionError
 *                           src/sim/kernels.cu:57-63, src/sim/monte_carlo.cu:324-333
 *   sw_prepare_params    <- parameters::prepare              src/sim/simulation_parameters.cuh:227-245
 *   sw_fieldmap_scale    <- Tesla -> degree-per-timestep factor src/sim/monte_carlo.cu:241
 *   sw_run_config        <- sim::monte_carlo::run            src/sim/monte_carlo.cu:199-355
 */
#ifndef SPINWALK_GPU_H
#define SPINWALK_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SW_ABI_VERSION 1

/* ---- return codes -------------------------------------------------------------------- */
#define SW_OK              0
#define SW_ERR_INVALID    -1   /* bad argument or inconsistent parameters */
#define SW_ERR_CUDA       -2   /* a CUDA runtime call failed */
#define SW_ERR_NOMEM      -3   /* device allocation failed or the HBM budget is exceeded */
#define SW_ERR_IO         -4   /* file could not be read or written */
#define SW_ERR_CONFIG     -5   /* config file rejected (same checks as config_reader::check) */
#define SW_ERR_TIMEOUT    -6   /* a bounded device loop gave up (reported, never a hang) */

/* ---- per-spin status (written to the optional `status` array) ------------------------ */
#define SW_SPIN_OK         0   /* walked to the end of the last scan */
#define SW_SPIN_LOST       1   /* more than max_iterations rejected moves in a row
                                  (reference: printf + return, src/sim/kernels.cu:155-158) */
#define SW_SPIN_OOB        2   /* voxel index outside the phantom
                                  (reference: printf + return, src/sim/kernels.cu:141-147) */
#define SW_SPIN_START_OOB  3   /* starting position outside the phantom (the reference reads
                                  mask[] out of bounds there, src/sim/kernels.cu:102-103) */

/* ---- precision of the Bloch part (the walk itself is always bit-exact FP64) ----------- */
#define SW_PREC_FP32       0   /* the reference's arithmetic: float phase sum, float Bloch */
#define SW_PREC_FP64       1   /* same walk, phase sum + rotations + relaxation in double */
#define SW_PREC_KAHAN      2   /* same walk, compensated (Kahan) float phase sum */
/* Generator flavour, OR-ed into the `precision` argument of every entry point:
 *   SW_RNG_MT19937 (0) -- the reference's CPU build: std::mt19937 + libstdc++
 *                         normal_distribution<float> (polar method) (kernels.cu:82-85);
 *   SW_RNG_MINSTD      -- the reference's CUDA build: thrust::minstd_rand +
 *                         thrust::normal_distribution<float> (inverse erfc, one draw per
 *                         deviate) + thrust::uniform_real_distribution<float>
 *                         (kernels.cu:76-80), with unfused arithmetic, i.e. as that build's host
 *                         (--use_cpu) path computes it; its GPU kernel differs from it only where
 *                         nvcc contracts a*b+c into fused multiply-adds. */
#define SW_RNG_MT19937     0x000
#define SW_RNG_MINSTD      0x100
#define SW_PREC_MASK       0x0ff
/* Fieldmap record, OR-ed into `precision` (sw_sim, sw_sim_device, sw_sim_batch, sw_sim_spins,
 * sw_sim_signal): SW_FIELD_BF16 packs the phantom as 4-byte voxel records, the field rounded to
 * bfloat16 (round to nearest even) beside the substrate label, instead of 8-byte records with the
 * float field -- half the phantom's device memory and gather bytes. Trajectories, substrates and
 * status are unchanged (the field only enters the phase); M1 is that of the float run on the
 * field rounded to bfloat16, which differs from the float field's by the stated error of
 * bench.py --field-bf16 (no counterpart in the reference, whose fieldmap is float). */
#define SW_FIELD_BF16      0x200

/*
 * Scalar simulation parameters. Field-for-field mirror of sim::parameters
 * (src/sim/simulation_parameters.cuh:176-186), with bools widened to int32 and size_t to
 * uint64 so the layout is the same on every platform. Values are AFTER parameters::prepare():
 * c/s hold cos/sin of RF_FA[0]; n_timepoints = TR_us / timestep_us.
 */
typedef struct sw_params {
    double   fov[3];                  /* field of view in m (after FoV scaling)           */
    float    B0;                      /* T (the fieldmap passed in is already deg/step)   */
    float    c, s;                    /* cosf/sinf(RF_FA_deg[0] * pi/180)                 */
    float    linear_phase_cycling;    /* degrees added to RF_PH[0] per dummy scan         */
    float    quadratic_phase_cycling; /* degrees, quadratic term                          */
    int32_t  timestep_us;
    int32_t  TR_us;
    int32_t  n_dummy_scan;
    uint32_t n_spins;
    uint32_t n_timepoints;
    uint32_t n_substrate;
    uint32_t n_scales;
    uint64_t phantom_size[3];         /* Nx, Ny, Nz; data are row-major, z fastest        */
    uint64_t seed;                    /* per-spin generators are seeded with seed + spin  */
    uint64_t max_iterations;          /* rejected moves allowed before a spin is lost     */
    int64_t  matrix_length;           /* Nx*Ny*Nz                                         */
    int32_t  enCrossFOV;              /* 1: periodic wrap, 0: reflect at the FoV boundary  */
    int32_t  enRecordTrajectory;      /* 1: XYZ1 holds every step, 0: final position only */
    int32_t  fieldmap_exist;
    int32_t  _pad;
} sw_params;

/*
 * Sequence and tissue tables. Mirror of parameters_uvec
 * (src/sim/simulation_parameters.cuh:102-106). Pointers are HOST pointers for sw_sim and
 * sw_sim_device alike (the library copies the tables itself). Times are in time points, i.e.
 * after config_reader::timing_scale (src/sim/config_reader.cpp:39-46), as in the reference.
 */
typedef struct sw_sequence {
    const double  *diffusivity;      /* [n_substrate] random-walk step std-dev in m        */
    const float   *T1_ms, *T2_ms;    /* [n_substrate]; negative = no relaxation            */
    const float   *pXY;              /* [n_substrate^2] crossing probability, row = from   */
    const float   *RF_FA_deg;        /* [n_RF]                                             */
    const float   *RF_PH_deg;        /* [n_RF]                                             */
    const int32_t *RF_us;            /* [n_RF] time points, RF_us[0] == 0                  */
    const int32_t *TE_us;            /* [n_TE] time points, strictly ascending             */
    const float   *dephasing_deg;    /* [n_dephasing]                                      */
    const int32_t *dephasing_us;     /* [n_dephasing] time points                          */
    const float   *gradientX_mTm;    /* [n_gradient]                                       */
    const float   *gradientY_mTm;
    const float   *gradientZ_mTm;
    const int32_t *gradient_us;      /* [n_gradient] time points                           */
    uint32_t n_RF, n_TE, n_dephasing, n_gradient;
} sw_sequence;

/*
 * Synthetic phantoms (host C++, OpenMP, deterministic per seed): uint8 mask (1 inside a shape)
 * and field in Tesla at B0 = 1 T, row-major [dims[0]][dims[1]][dims[2]]. The field models are
 * those of the reference's phantom generators (src/phantom/phantom_cylinder.cpp:255-265,
 * src/phantom/phantom_sphere.cpp:180-187); the placement differs (random orientations allowed,
 * overlaps allowed, sphere fields summed within +-window*r). `field` may be NULL.
 */
int sw_phantom_cylinders(const uint32_t dims[3], const double fov[3], double radius,
                         double volume_fraction, uint64_t seed, int random_orientation,
                         double dchi, double Y, const double B0_dir[3], uint8_t *mask,
                         float *field);
int sw_phantom_spheres(const uint32_t dims[3], const double fov[3], double rmin, double rmax,
                       double volume_fraction, uint64_t seed, double dchi, double Y,
                       const double B0_dir[3], double window, uint8_t *mask, float *field);

/*
 * Parses an INI config exactly as the reference's config_reader::prepare does (PARENT_CONFIG,
 * indexed keys, float-parsed vectors, checks, microseconds -> time points;
 * src/sim/config_reader.cpp:25-324) and writes the result as `key value...` text lines.
 * Returns SW_ERR_CONFIG when the reader rejects the file (the dump then holds "ok 0").
 */
int sw_config_dump(const char *ini_path, const char *out_path);

/*
 * sim::monte_carlo::run (src/sim/monte_carlo.cu:199-355) for one INI config on `device`: for
 * every PHANTOM: read the HDF5 phantom (mask, fieldmap, fov), the optional XYZ0 file, scale the
 * fieldmap to degrees per time step, run every SCALE, and write the result file
 * OUTPUT_DIR/SEQ_NAME_<phantom>.h5 with datasets M, XYZ, T, scales, TE as the reference does.
 */
int sw_run_config(const char *ini_path, int device);

/* Whole-dataset HDF5 I/O (root group; little-endian, contiguous or compact): the subset
 * SpinWalk's phantom and result files use. Type codes: uint8 = 0, float32 = 1, float64 = 2,
 * int8 = 3, uint16 = 4, int16 = 5, uint32 = 6, int32 = 7, uint64 = 8, int64 = 9. sw_h5_read
 * returns the stored type and bytes (with out == NULL only type, rank and dims); sw_run_config
 * converts what it reads to the types the reference reads (mask uint8, the rest float) as
 * libhdf5 does: integers saturate, floats truncate toward zero (NaN -> 0). */
int sw_h5_write(const char *path, int n, const char *const *names, const int *types,
                const int *ranks, const uint64_t *dims, const void *const *data);
int sw_h5_read(const char *path, const char *name, int *type, int *rank, uint64_t dims[8],
               void *out, uint64_t out_bytes);

/* Library and device information. */
int         sw_abi_version(void);
const char *sw_last_error(void);
int         sw_device_count(int *count);
/* sim::print_device_info (src/sim/device_helper.cu:47-76), the CLI's -g/--gpu_info, as text in
 * `buf` (NUL-terminated, at most `len` bytes): the CUDA versions of driver and runtime, the
 * number of devices, and for `device` its name, compute capability and free / total memory.
 * Without a device the text says so and SW_ERR_CUDA is returned. */
int         sw_device_info(int device, char *buf, uint64_t len);

/*
 * parameters::prepare (src/sim/simulation_parameters.cuh:227-245) on plain arrays:
 * sets c/s from RF_FA_deg[0], n_timepoints = TR/dt, replaces seed 0 by a random seed,
 * converts diffusivity[i] (m^2/s, in place) to the step std-dev 1e-3*sqrt(2*D*dt_us), and
 * sets n_dummy_scan = 5*T1[0]/TR when it is negative.
 */
int sw_prepare_params(sw_params *p, double *diffusivity, const float *RF_FA_deg,
                      const float *T1_ms);

/* Factor from Tesla (at 1 T) to degree per time step, computed as the reference does
 * (src/sim/monte_carlo.cu:241): float(B0*dt*1e-6*GAMMA*RAD2DEG). */
float sw_fieldmap_scale(float B0, int32_t timestep_us);

/* Initial positions when no XYZ0 file is given: monte_carlo::initialize_position
 * (src/sim/monte_carlo.cu:141-151): std::mt19937(seed), per spin x, y, z drawn from
 * uniform_real_distribution<float>(0.01*fov, 0.99*fov). XYZ0 is [n_spins*3]. */
int sw_initial_positions(const float fov[3], uint64_t seed, uint32_t n_spins, float *XYZ0);

/* Size of the table that makes the device logf equal to this host's libm logf (built on first
 * use; `wide` counts differences larger than one ulp and must be 0). No reference counterpart:
 * it exists so that the GPU reproduces libstdc++'s normal_distribution<float> bit for bit. */
int sw_logf_exception_count(uint64_t *count, uint64_t *wide);

/*
 * Run the whole walk for all p->n_spins spins of ONE scale, host buffers in and out.
 * Replaces the per-scale CPU loop std::for_each(par_unseq, sim(...)) of
 * src/sim/monte_carlo.cu:313-321 with the GPU kernels; semantics are those of sim::sim
 * (src/sim/kernels.cu:72-233) with the libstdc++ std::mt19937 generators, bit for bit.
 *   pFieldMap : [matrix_length] float, degree per time step, or NULL (no off-resonance)
 *   pMask     : [matrix_length] uint8 substrate index
 *   M0, XYZ0  : [n_spins*3] float
 *   M1        : [n_spins*n_TE*3]  written at echo times only (untouched for echoes a lost
 *               or out-of-bounds spin never reaches, as in the reference)
 *   XYZ1      : [n_spins*(enRecordTrajectory ? (n_dummy_scan+1)*n_timepoints : 1)*3]
 *   T         : [n_spins*n_TE] substrate at each echo
 *   status    : [n_spins] SW_SPIN_* or NULL
 *   precision : SW_PREC_*; M1_fp64 (optional, [n_spins*n_TE*3] double) receives the FP64
 *               shadow magnetisation of the same walk when non-NULL.
 * The GPU starts seeding the generators before the buffers are copied in (seeding reads none
 * of them), so the copies overlap it; pinned host buffers copy fastest. The device workspace
 * and the device copies of the buffers are kept per device for the next call, grown on demand.
 */
int sw_sim(const sw_params *param, const sw_sequence *seq,
           const float *pFieldMap, const uint8_t *pMask,
           const float *M0, const float *XYZ0,
           float *M1, float *XYZ1, uint8_t *T, int32_t *status,
           int precision, double *M1_fp64);

/* Same as sw_sim with DEVICE buffers (the cu_sim analogue). The walk is ordered after the work
 * already on `stream` (which may still be producing the inputs); the seeding, which reads none
 * of them, starts at once beside it. The call returns once its own work has finished: between
 * refill/walk rounds the host reads how many spins are still walking. */
int sw_sim_device(const sw_params *param, const sw_sequence *seq,
                  const float *d_FieldMap, const uint8_t *d_Mask,
                  const float *d_M0, const float *d_XYZ0,
                  float *d_M1, float *d_XYZ1, uint8_t *d_T, int32_t *d_status,
                  int precision, double *d_M1_fp64, void *stream);
int sw_sync(void *stream);

/*
 * Many instances of one configuration that walk identically, in one pass: the reference's
 * phase-cycling scales (WHAT_TO_SCALE = 2, src/sim/monte_carlo.cu:302-305), its DUMMY_SCAN
 * sweeps and per-pulse flip-angle / phase variants all re-run the same trajectories (same seeds,
 * same XYZ0; the scan structure does not touch the random streams). sw_sim_tracks walks every
 * spin ONCE and advances one Bloch state per distinct RF configuration; each track's outputs
 * are bit-identical to sw_sim on that instance alone.
 *
 * A track = one instance: its phase cycling, its DUMMY_SCAN (echoes are recorded in that
 * scan), optional per-pulse RF_FA / RF_PH arrays (NULL = the sequence's), and host output
 * buffers. `param` supplies everything else (its n_dummy_scan, phase cycling, c and s are
 * ignored; enRecordTrajectory must be 0). Tracks with identical RF configuration and
 * DUMMY_SCAN are rejected as duplicates.
 *
 * precision : SW_PREC_FP32 (the reference's arithmetic), SW_PREC_KAHAN (compensated float phase
 * sums) or SW_PREC_FP64 (M1 = the FP64 values rounded to float), as for sw_sim. A track's M1_fp64
 * (optional, host [n_spins][n_TE][3]) receives the FP64 shadow of that track: the steady-state
 * recurrence over all DUMMY_SCAN scans carried in double, bit-identical to sw_sim's M1_fp64 on
 * that instance. SW_RNG_MINSTD and SW_FIELD_BF16 may be OR-ed in, as for sw_sim.
 */
typedef struct sw_track {
    float linear_phase_cycling;
    float quadratic_phase_cycling;
    int32_t n_dummy_scan;
    int32_t _pad;
    const float *RF_FA_deg;   /* [n_RF] or NULL */
    const float *RF_PH_deg;   /* [n_RF] or NULL */
    float *M1;                /* [n_spins][n_TE][3] host */
    float *XYZ1;              /* [n_spins][3] host: final position */
    uint8_t *T;               /* [n_spins][n_TE] host */
    int32_t *status;          /* [n_spins] host, or NULL */
    double *M1_fp64;          /* [n_spins][n_TE][3] host FP64 shadow, or NULL */
    float gradient_scale;     /* with SW_TRACK_GRADIENT_SCALE: the gradients times this scale */
    uint32_t options;         /* SW_TRACK_* bits */
} sw_track;
/* The track's gradient waveform is the sequence's scaled by gradient_scale (float multiply, as
 * the reference's gradient scale loop does, src/sim/monte_carlo.cu:287-290). Tracks with
 * different gradient scales share the walk but not the phase: each distinct scale keeps its own
 * phase sums (at most 8 distinct scales per call; SW_PREC_FP32 or _KAHAN, no FP64 shadow). */
#define SW_TRACK_GRADIENT_SCALE 0x1u

int sw_sim_tracks(const sw_params *param, const sw_sequence *seq, const sw_track *tracks,
                  uint32_t n_tracks, const float *pFieldMap, const uint8_t *pMask,
                  const float *M0, const float *XYZ0, int precision);

/*
 * sw_sim_device without any device allocation, for callers that are not allowed to allocate
 * device memory: a process whose device memory is reserved up front by a pool or another
 * framework's allocator, a real-time loop that cannot take cudaMalloc's implicit device-wide
 * synchronisation, or a host application that forbids libraries from allocating on their own.
 * No counterpart in the reference (its driver allocates thrust device_vectors per run).
 *
 * The caller passes device inputs and outputs exactly as for sw_sim_device (FP32 precision, no
 * FP64 shadow). All other device memory comes from one static array of SW_NOALLOC_SCRATCH_BYTES
 * that every GPU loading this part of the library keeps until the process exits. About 48 MiB of
 * it hold the logf correction table; the rest must fit the call: roughly 8.5 KiB per spin plus
 * 8 bytes per voxel -- larger requests are rejected with SW_ERR_NOMEM and a message, never
 * partially run. No cudaMalloc/cudaFree or other device-allocating routine is called (host-side
 * staging of the small parameter tables uses ordinary host memory).
 *
 * The first call on a device sets the region up (resolves the array's device address and copies
 * the logf table into it, synchronously); make that first call before any stream capture. Every
 * call reuses the same array and finds the previous call's contents there; it re-initialises all
 * state it reads. Calls on one device are serialised by the library and each returns only after
 * its work on `stream` has finished; any other work that touched the array while a call runs on
 * the GPU would race with it.
 */
#define SW_NOALLOC_SCRATCH_BYTES (128ull << 20)
int sw_sim_device_noalloc(const sw_params *param, const sw_sequence *seq,
                          const float *d_FieldMap, const uint8_t *d_Mask,
                          const float *d_M0, const float *d_XYZ0,
                          float *d_M1, float *d_XYZ1, uint8_t *d_T, int32_t *d_status,
                          void *stream);

/* Frees what the one-call entry points keep on the current device between calls: the device
 * workspaces of sw_sim / sw_sim_device (generator state, rings, walk state), sw_sim's device
 * copies of the caller's buffers, the pooled batch's workspace and pinned staging, and the
 * internal engine of sw_sim_batch / sw_sim_spins / sw_sim_signal. They are otherwise kept until
 * the process exits, grown to the largest call so far (about 12 KB per spin). The next call
 * allocates again. Waits for a call running on another thread to finish; engines created with
 * sw_engine_create, the logf table and the minstd deviate table are not touched. No counterpart
 * in the reference (its driver frees its thrust vectors after every scale). */
int sw_release_workspaces(void);

/* Timing of the kernels launched by the last sw_sim / sw_sim_device call on this thread
 * (milliseconds, CUDA events on the launching stream): seeding, RNG refill, walk, total. After
 * sw_sim_batch with pooled generators: seed_ms the seeding of the streams, walk_ms all rounds
 * (refills and walks together), refill_ms 0, total_ms the call's wall time. */
typedef struct sw_timing {
    float seed_ms, refill_ms, walk_ms, total_ms;
    uint32_t n_chunks;       /* refill+walk rounds                                   */
    uint32_t n_launches;     /* kernels launched by the call                         */
} sw_timing;
int sw_last_timing(sw_timing *out);

/*
 * Walk tuning, process-wide: read at the start of every later call (sw_sim, sw_sim_device,
 * sw_sim_batch, sw_sim_spins, sw_sim_signal, engine chunks). Results never depend on it: it only
 * changes which thread walks which spin and the walk kernel's block size. No counterpart in the
 * reference (one thread per spin in id order, src/sim/kernels.cu:70-90).
 *   resort_interval : refill/walk rounds (256 steps each) between Morton re-sorts of the spins
 *                     by their current voxel; 0 = never (id order)
 *   walk_block      : threads per block of the walk kernel: 64, 128 or 256
 *   seed_chunks     : sw_sim / sw_sim_device seed the spins in this many chunks of equal seeding
 *                     cost on a low-priority stream and walk each seeded chunk on a
 *                     high-priority stream meanwhile (0 or 1 = seed everything, then walk; at
 *                     most 64). It pays only where the walk is a sizeable share of the discards
 *                     (8 chunks on 1e6 spins of 2001 steps: 1.4 % faster); elsewhere the
 *                     co-resident kernels slow each other down by more than the overlap saves.
 *   round_streams   : sw_sim / sw_sim_device run the refill/walk rounds of the spins as this
 *                     many independent halves on their own streams (1 = one, 2 = two, 0 = auto:
 *                     two from 2^17 spins on), so that one half's walk overlaps the other
 *                     half's refill
 *   jump_min_kwords : seeding: spins whose discard count seed + spin reaches this many times
 *                     1024 words compute their state by jump-ahead (a polynomial over GF(2),
 *                     work independent of the count) instead of generating seed + spin words;
 *                     0 = default (1408, i.e. 1.44e6 words, where the two cost the same on
 *                     GB300). No reference counterpart (the reference discards word by word,
 *                     src/sim/kernels.cu:87-88).
 *   ring_steps      : sw_sim / sw_sim_device / sw_sim_spins / sw_sim_signal and the slots of
 *                     engines created afterwards (sw_engine_create; sw_sim_batch instances that
 *                     run as engine jobs): walk steps one refill of a spin's Gaussian ring
 *                     lasts (3 deviates each), i.e. the steps of one refill/walk round and of
 *                     one walk launch; 0 = default (512), else 32 .. 4096. Longer rings mean
 *                     fewer rounds and launches but more ring memory (12 B per step per spin)
 *                     between refill and walk.
 *   walk_blocks_per_sm : sw_sim / sw_sim_device: caps the walk launch at this many blocks per
 *                     SM, the blocks striding over the spins, so that the other half's refill
 *                     can run beside it on every SM; sw_sim_batch (pooled generators): the
 *                     fused walk over all instances then runs as persistent blocks striding over
 *                     the instances' blocks; 0 = default (no cap, one thread per spin).
 */
typedef struct sw_tuning {
    uint32_t resort_interval;
    uint32_t walk_block;
    uint32_t seed_chunks;
    uint32_t round_streams;
    uint32_t jump_min_kwords;
    uint32_t ring_steps;
    uint32_t walk_blocks_per_sm;
    uint32_t reserved[1];
} sw_tuning;
int sw_set_tuning(const sw_tuning *t);
int sw_get_tuning(sw_tuning *t);

/* One measured candidate of sw_autotune: device time of the refill and walk per 256 walk steps,
 * the re-sorts' share included (model: (sort + sum of the rounds at age 0..I-1 after a sort) / I),
 * rounds of ring_steps steps scaled to 256. */
typedef struct sw_tune_entry {
    uint32_t resort_interval;
    uint32_t walk_block;
    float ms_per_round;
    float sort_ms;            /* one re-sort (0 for resort_interval 0) */
    uint32_t ring_steps;      /* steps of one refill/walk round */
} sw_tune_entry;

/*
 * Picks the fastest sw_tuning for the walk of this problem by a probe on the current device: the
 * problem's phantom, spin count, start positions and tissue, walked for up to 20 rounds (time
 * points extended, no dummy scans, generators of the SW_RNG_MINSTD flavour because their seeding
 * costs O(log) per spin and the walk is the same), timing every round with CUDA events. Candidates:
 * resort_interval in {0, 1, 2, 4, 8} x walk_block in {128, 256} with rounds of 256 steps, and
 * rounds of 128 or 512 steps (ring_steps) in id order at block 256. `best` receives the fastest;
 * `table` (optional, table_len entries) the measured candidates, *n_entries their number;
 * apply != 0 installs `best` with sw_set_tuning. The probe allocates its own device memory
 * (about as much as sw_sim on the problem) and frees it before returning.
 */
int sw_autotune(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
                const uint8_t *pMask, const float *XYZ0, int apply, sw_tuning *best,
                sw_tune_entry *table, uint32_t table_len, uint32_t *n_entries);

/* One instance of a batch: its parameters, sequence and host buffers, as for sw_sim. */
typedef struct sw_instance {
    const sw_params *param;
    const sw_sequence *seq;
    const float *M0, *XYZ0;  /* [n_spins][3] */
    float *M1;               /* [n_spins][n_TE][3] */
    float *XYZ1;             /* [n_spins][traj][3] */
    uint8_t *T;              /* [n_spins][n_TE] */
    int32_t *status;         /* optional [n_spins] */
} sw_instance;

/* Several instances on one phantom, e.g. the FoV- or gradient-scaled instances of
 * monte_carlo::run's scale loop (src/sim/monte_carlo.cu:273-337) or instances with different
 * sequences or spin counts. Every instance gives the same results as its own sw_sim call; the
 * batch uploads and packs the phantom once and seeds the generators once: the state of spin s
 * depends only on seed + s (src/sim/kernels.cu:82-88), so the instances (which must share the
 * seed, phantom size, substrate count and fieldmap) start from prefixes of one seeding of the
 * largest instance. pFieldMap is in degrees per time step (already scaled, as for sw_sim).
 * With the std::mt19937 generators, instances also share one Gaussian stream per spin id, and
 * every refill/walk round is one launch of each kernel over all instances, replayed as a CUDA
 * graph; above half the free device memory, and with SW_RNG_MINSTD, the instances run as jobs
 * of an internal serving engine instead. No reference counterpart: the reference re-seeds every
 * spin for every scale. */
int sw_sim_batch(const sw_instance *items, uint32_t n_items, const float *pFieldMap,
                 const uint8_t *pMask, int precision);

/* Spins [spin_lo, spin_hi) of one sw_sim call, for sharding a job across GPUs or processes:
 * M0, XYZ0, M1, XYZ1, T and status hold the rows of those spins only (row 0 = spin_lo); the
 * results equal those rows of the full call bit for bit (a spin's generators and walk depend
 * only on its id). Only the range's generator states are seeded. No reference counterpart (the
 * reference's per-spin function sim::sim(..., spin_no), src/sim/kernels.cuh:21-30, is the
 * one-spin case). */
int sw_sim_spins(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
                 const uint8_t *pMask, const float *M0, const float *XYZ0, uint32_t spin_lo,
                 uint32_t spin_hi, float *M1, float *XYZ1, uint8_t *T, int32_t *status,
                 int precision);

/* ---- Engine: many jobs on one GPU (scale sweeps, serving) --------------------------------
 * No reference counterpart: the reference runs one job at a time (monte_carlo::run). An engine
 * keeps phantoms resident (packed once), seeds each simulation seed's generator states once for
 * all its jobs (the state of spin s depends only on seed + s, src/sim/kernels.cu:82-88), and runs
 * jobs in spin-range chunks on `n_slots` concurrent slots of `slot_spins` spins each (about
 * 6.4 KB of device memory per slot spin, plus a 256 B-per-spin I/O buffer). Every job gives the
 * results of its own sw_sim call, bit for bit. hbm_budget = 0: 85 % of the free device memory;
 * phantoms that no queued job uses are evicted when a new one does not fit. One host thread
 * drives an engine; its host buffers must stay valid until the job is reported done. */
typedef struct sw_engine sw_engine;
typedef struct sw_job_result {
    int64_t job_id;
    int32_t rc;              /* SW_OK or the job's error                                */
    int32_t _pad;
    double latency_s;        /* submit -> results in the caller's buffers               */
} sw_job_result;

int sw_engine_create(int device, uint32_t n_slots, uint32_t slot_spins, uint64_t hbm_budget,
                     sw_engine **out);
int sw_engine_destroy(sw_engine *e);
/* mask u8 and optional field (degrees per time step, i.e. already scaled as for sw_sim) of
 * dims[0] x dims[1] x dims[2] voxels, z fastest */
int sw_engine_add_phantom(sw_engine *e, const uint8_t *mask, const float *field_deg_per_step,
                          const uint64_t dims[3], uint32_t n_substrate, int32_t *phantom_id);
/* as sw_engine_add_phantom; flags = SW_FIELD_BF16 packs 4-byte records (jobs on the phantom then
 * run with the bfloat16 field; a job that passes SW_FIELD_BF16 needs such a phantom) */
int sw_engine_add_phantom_ex(sw_engine *e, const uint8_t *mask, const float *field_deg_per_step,
                             const uint64_t dims[3], uint32_t n_substrate, int flags,
                             int32_t *phantom_id);
/* queues one job (the arguments of sw_sim, on a registered phantom); nothing runs until
 * sw_engine_poll */
int sw_engine_submit(sw_engine *e, int32_t phantom, const sw_params *param, const sw_sequence *seq,
                     int precision, const float *M0, const float *XYZ0, float *M1, float *XYZ1,
                     uint8_t *T, int32_t *status, int64_t *job_id);
/* Advances the work and reports finished jobs (at most max_done). wait: 0 = one non-blocking
 * pass, 1 = until a job finishes or nothing is queued, 2 = until nothing is queued. */
int sw_engine_poll(sw_engine *e, int wait, sw_job_result *done, uint32_t max_done,
                   uint32_t *n_done);
int sw_engine_pending(sw_engine *e, uint32_t *n_pending);
/* Counters since sw_engine_create: kernels launched, refill/walk rounds issued, seedings; and
 * the device memory the engine holds against its HBM budget (slots, resident phantoms, seed
 * caches), with the number of seed caches held. Seed caches that no queued job uses are freed,
 * least recently used first, when a new one would exceed the budget. */
typedef struct sw_engine_stats {
    uint64_t launches;
    uint64_t rounds;
    uint64_t seedings;
    uint64_t hbm_used;
    uint64_t hbm_budget;
    uint64_t seed_caches;
} sw_engine_stats;
int sw_engine_get_stats(sw_engine *e, sw_engine_stats *out);

/* ---- Signal mode: the reduction of the results fused into the walk ------------------------
 * What the reference's analysis computes from M1 and T (the demos average M per tissue and
 * echo) without writing them: signal[te][substrate][0..2] = the sum over spins of M at echo
 * te of the spins in that substrate at the echo, count[te][substrate] = how many spins (spins
 * lost or out of bounds before an echo are not in that echo's sums). Sums in double; the order
 * of the additions is not fixed, so results agree with a reduction of sw_sim's M1 / T to about
 * 1e-15 relative. XYZ1 is not produced. No reference counterpart. */
int sw_sim_signal(const sw_params *param, const sw_sequence *seq, const float *pFieldMap,
                  const uint8_t *pMask, const float *M0, const float *XYZ0, double *signal,
                  uint64_t *count, int32_t *status, int precision);
int sw_engine_submit_signal(sw_engine *e, int32_t phantom, const sw_params *param,
                            const sw_sequence *seq, int precision, const float *M0,
                            const float *XYZ0, double *signal, uint64_t *count, int32_t *status,
                            int64_t *job_id);


/* ---- The reference's phantom generators, mask and field on the GPU -----------------------
 * phantom::cylinder (src/phantom/phantom_cylinder.cpp: parallel cylinders along z, B0 rotated
 * by `orientation_deg` about y) and phantom::sphere (phantom_sphere.cpp), with the reference's
 * arguments and units: fov in um, `resolution` voxels per side, dChi, Y (< 0: no field),
 * radius in um (< 0: random radii up to |radius|), volume fraction in percent, seed. Outputs:
 * mask u8 and field f32 (T at B0 = 1 T; may be NULL) of resolution^3 voxels, z fastest, and the
 * actual volume fraction. Shapes are placed on the host as the reference does; mask and field
 * are bit-identical to the reference's (with random radii: to the reference run on one
 * thread). The _device variants take device buffers (e.g. for sw_engine_add_phantom). */
int sw_phantom_cylinder(float fov_um, uint64_t resolution, float dchi, float Y, float radius_um,
                        float volume_fraction, float orientation_deg, int32_t seed, uint8_t *mask,
                        float *field, float *bvf_out);
int sw_phantom_sphere(float fov_um, uint64_t resolution, float dchi, float Y, float radius_um,
                      float volume_fraction, int32_t seed, uint8_t *mask, float *field,
                      float *bvf_out);
int sw_phantom_cylinder_device(float fov_um, uint64_t resolution, float dchi, float Y,
                               float radius_um, float volume_fraction, float orientation_deg,
                               int32_t seed, uint8_t *d_mask, float *d_field, float *bvf_out);
int sw_phantom_sphere_device(float fov_um, uint64_t resolution, float dchi, float Y,
                             float radius_um, float volume_fraction, int32_t seed,
                             uint8_t *d_mask, float *d_field, float *bvf_out);

/* Host-visible check of the bit-exact logf used by the Gaussian generator: evaluates the
 * device logf on n inputs (device pointers) -- used by the tests. */
int sw_debug_logf(const float *d_x, float *d_y, uint64_t n, void *stream);

/* Host-visible check of the minstd flavour's Gaussian deviate (thrust normal_distribution_nvcc,
 * device erfcinvf): d_y[i] = deviate of engine output x_lo + i -- used by the tests. */
int sw_debug_ms_normal(uint32_t x_lo, uint32_t n, float *d_y, void *stream);

/* Host-visible check of the integer double addition of the walk's position update:
 * d_y[i] = d_a[i] + d_b[i] (IEEE round to nearest even) on n device doubles -- used by the
 * tests. */
int sw_debug_dadd(const double *d_a, const double *d_b, double *d_y, uint64_t n, void *stream);

/* Host-visible check of the walk's gradient-phase arithmetic: d_y[i] = (float)d_x[i] (round to
 * nearest even) by the integer conversion the walk uses, on n device doubles -- used by the
 * tests. */
int sw_debug_d2f(const double *d_x, float *d_y, uint64_t n, void *stream);

/* Host-side check of the jump-ahead seeding (no GPU needed): the state of std::mt19937(z) after
 * discard(z) -- its 624-word buffer and next position -- computed through the jump polynomial
 * that the seeding kernel uses for large discard counts. No reference counterpart (the
 * reference discards word by word, src/sim/kernels.cu:87-88) -- used by the tests. */
int sw_debug_mt_jump(uint64_t z, uint32_t *block, uint32_t *pos);

#ifdef __cplusplus
}
#endif
#endif /* SPINWALK_GPU_H */
