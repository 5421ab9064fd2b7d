/*
 * gpl.h - C ABI of the GB300 global-placement core (libgpl_gb300.so).
 *
 * The library is a drop-in for RePlAce's electrostatic global placement:
 * the initial place (B2B + BiCGSTAB) and the Nesterov loop.  Each entry point
 * below names the reference interface it replaces (paths are relative to the
 * RePlAce source tree).  Signatures use plain C types and pointers only.
 *
 * Ownership: every pointer argument is caller-owned host memory that is read
 * (or written) during the call only, unless the comment says "device".  A job
 * owns all the device memory it allocates; gpl_destroy releases it.
 * Threading: one job must not be used from two threads at once; distinct jobs
 * are independent.  Errors: every call returns a gpl_status; the reference's
 * Logger::error exit codes (src/logger.cpp:31-36) become status values with
 * the same numbers, and gpl_last_error() gives the message.  Nothing here
 * calls exit().
 */
#ifndef GPL_GB300_GPL_H
#define GPL_GB300_GPL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GPL_ABI_VERSION 1

typedef enum gpl_status {
  GPL_OK = 0,
  /* Negative filler area: NesterovBase::initFillerGCells, code 1
   * (src/nesterovBase.cpp:1116-1121). */
  GPL_ERR_FILLER_AREA = 1,
  /* NaN/Inf gradient sums during NesterovPlace::init, code 2
   * (src/nesterovPlace.cpp:280-284). */
  GPL_ERR_DIVERGED_INIT = 2,
  /* Back-tracking ran out (maxBackTrack), code 3 (src/nesterovPlace.cpp:404-409). */
  GPL_ERR_DIVERGED_BACKTRACK = 3,
  /* Overflow went up while HPWL blew up, code 4 (src/nesterovPlace.cpp:448-456). */
  GPL_ERR_DIVERGED_PHI = 4,
  /* Placeable area above 100.1 % of free core area: PlacerBase::printInfo
   * exits with 1 (src/placerBase.cpp:952-956). */
  GPL_ERR_UTIL = 5,
  /* NaN/Inf gradient sums inside the Nesterov loop; the reference reports
   * this through Logger::error with code 0 (src/nesterovPlace.cpp:371-374,
   * 469-471). */
  GPL_ERR_DIVERGED_NAN = 6,
  GPL_ERR_INVALID_ARG = 16,
  GPL_ERR_CUDA = 17,
  GPL_ERR_OUT_OF_MEMORY = 18,
  GPL_ERR_BAD_STATE = 19,
  GPL_ERR_NO_DEVICE = 20,
  /* A server job cancelled before it finished (gpl_server_cancel). */
  GPL_ERR_CANCELLED = 21
} gpl_status;

/* Instance kinds (PlacerBase::init, src/placerBase.cpp:639-680). */
enum {
  GPL_INST_PLACE = 0,    /* movable */
  GPL_INST_FIXED = 1,    /* fixed, overlaps the core */
  GPL_INST_DUMMY = 2,    /* fragmented-row dummy (initInstsForFragmentedRow) */
  GPL_INST_OUTSIDE = 3   /* fixed, outside the core: ignored */
};

/*
 * Flat netlist: the data PlacerBase (src/placerBase.h:233-312) builds from
 * OpenDB.  Pins are net-major: net n owns pins [net_start[n], net_start[n+1]).
 * Within a net, component pins come first, then IO pins, in
 * dbNet::getITerms / getBTerms order.
 */
typedef struct gpl_netlist_desc {
  int32_t core_lx, core_ly, core_ux, core_uy;   /* rows' bounding box */
  int32_t site_w, site_h;
  int32_t n_insts;
  const int32_t* inst_lx;      /* [n_insts] bounding boxes (DBU) */
  const int32_t* inst_ly;
  const int32_t* inst_ux;
  const int32_t* inst_uy;
  const uint8_t* inst_kind;    /* GPL_INST_* */
  int32_t n_pins;
  const int32_t* pin_inst;     /* [n_pins] instance index, -1 for an IO port */
  const int32_t* pin_ox;       /* offset of the pin centre from the instance centre */
  const int32_t* pin_oy;
  const int32_t* pin_x;        /* initial absolute pin centre */
  const int32_t* pin_y;
  int32_t n_nets;
  const int32_t* net_start;    /* [n_nets + 1] */
  /* Optional per-instance pin order (dbInst::getITerms); NULL = ascending
   * pin index.  [n_insts + 1] and [number of component pins]. */
  const int32_t* inst_pin_start;
  const int32_t* inst_pins;
} gpl_netlist_desc;

/* Placement parameters: the members of replace::Replace
 * (include/replace/Replace.h:75-93) plus the hidden InitialPlaceVars,
 * NesterovBaseVars and NesterovPlaceVars fields, plus GB300 knobs. */
typedef struct gpl_params {
  /* InitialPlaceVars (src/initialPlace.h:12-23) */
  int32_t initial_place_max_iter;          /* 20 */
  int32_t initial_place_min_diff_length;   /* 1500 */
  int32_t initial_place_max_solver_iter;   /* 100 */
  int32_t initial_place_max_fanout;        /* 200 */
  float initial_place_net_weight_scale;    /* 800 */
  int32_t incremental_place_mode;          /* 0 */
  /* NesterovBaseVars (src/nesterovBase.h:695-708) */
  float target_density;                    /* 1.0 (Replace); the Tcl default is 0.7 */
  int32_t bin_grid_cnt_x;                  /* 0 = bin-count rule */
  int32_t bin_grid_cnt_y;
  float min_wire_length_force_bar;         /* -300 */
  /* NesterovPlaceVars (src/nesterovPlace.h:16-29) */
  int32_t nesterov_place_max_iter;         /* 2000 */
  int32_t max_back_track;                  /* 10 */
  float init_density_penalty;              /* 0.00008 */
  float init_wire_length_coef;             /* 0.25 */
  float target_overflow;                   /* 0.1 */
  float min_phi_coef;                      /* 0.95 */
  float max_phi_coef;                      /* 1.05 */
  float min_preconditioner;                /* 1.0 */
  float initial_prev_coordi_update_coef;   /* 100 */
  float reference_hpwl;                    /* 446000000 */
  int32_t verbose_level;                   /* 0: print the reference's default log lines */
  /* GB300 knobs */
  int32_t device;                          /* CUDA device ordinal */
  void* stream;                            /* cudaStream_t to run on; NULL = job-owned stream */
  int32_t use_graph;                       /* 1 = each evaluation replays one CUDA graph */
  int32_t ip_solver;                       /* BiCGSTAB form: 0 = auto (= 1), 1 = one kernel
                                              per phase, 2 = one cooperative grid launch per
                                              solve (same iterates as 1), 3 = one thread-block
                                              cluster per axis (up to 65536 instances) */
  int32_t poisson_path;                    /* Poisson solve: 0 = auto (times both forms on the job's
                                              grid and keeps the faster; the GEMM form only up to
                                              512 bins per axis, where it can be the faster: larger
                                              grids keep the FFT form untimed), 1 = FFT (register
                                              FFTs per warp on 512^2 and 1024^2 grids, shared-memory
                                              FFTs otherwise), 2 = tensor-core GEMMs (each value
                                              split into three bf16 terms, six products per GEMM;
                                              grids with both counts multiples of 128) */
  int32_t scatter_tile;                    /* scatter tile side in bins (16, 32 or 64); 0 = chosen
                                              by timing at gpl_nesterov_init */
  int32_t scatter_chunk;                   /* gcells per scatter block (1024 or 2048); 0 = chosen
                                              by timing (with the tile) */
  int32_t device_loop;                     /* 0 = the host drives the Nesterov loop, one
                                              evaluation graph at a time, and the initial
                                              place's rounds, one chunk of solver iterations
                                              at a time (default); 1 = both run on the device
                                              (CUDA graphs with conditional WHILE nodes and
                                              one-thread control kernels).  Same control
                                              arithmetic and results; the host-driven form
                                              interleaves better with other jobs' work. */
} gpl_params;

/* Counts and grid chosen by the job (NesterovBase / BinGrid). */
typedef struct gpl_job_info {
  int32_t n_place_insts;
  int32_t n_gcells;          /* movable instances followed by fillers */
  int32_t n_fillers;
  int32_t bin_cnt_x, bin_cnt_y;
  int32_t bin_size_x, bin_size_y;
  int32_t filler_dx, filler_dy;
  int64_t place_insts_area, std_insts_area, macro_insts_area, non_place_insts_area;
  int64_t device_bytes;      /* device memory held by the job */
  int32_t poisson_path;      /* the form the job runs: 1 FFT, 2 tensor-core GEMMs */
  float poisson_fft_us;      /* the timings auto mode compared (0 if not timed) */
  float poisson_gemm_us;
  int32_t scatter_tile;      /* the scatter's tile side in bins, chosen by timing (16, 32 or 64) */
  int32_t scatter_chunk;     /* gcells per scatter block, chosen with the tile */
  float scatter_us;          /* the chosen shape's scatter time */
} gpl_job_info;

/* One physics evaluation (the work of NesterovBase for one coordinate set). */
typedef struct gpl_eval_stats {
  int64_t overflow_area;     /* FP64-accumulated sum of max(0, inst+nonPlace-binArea*td), truncated */
  double overflow_area_f64;
  int64_t hpwl;              /* NesterovBase::getHpwl, exact int64 */
  double sum_phi;            /* FP64 sum of phi * (nonPlace+inst+filler) */
  double wire_length_grad_sum;   /* sum |dWL/dx| + |dWL/dy| (FP64) */
  double density_grad_sum;       /* sum |dD/dx| + |dD/dy| (FP64) */
} gpl_eval_stats;

/* Nesterov progress (NesterovPlace::doNesterovPlace). */
typedef struct gpl_nesterov_stats {
  int32_t iterations;        /* iterations completed so far */
  int32_t evaluations;       /* physics evaluations (back-track tries) so far */
  int32_t finished;          /* 1 when the loop stopped (converged or diverged) */
  int32_t status;            /* gpl_status of the loop: GPL_OK or a divergence code */
  float overflow;            /* sumOverflow_ */
  float step_length;
  float density_penalty;
  float wire_length_coef;
  int64_t hpwl;              /* prevHpwl_ */
} gpl_nesterov_stats;

/* Optional per-iteration log (may be NULL); the call appends up to capacity. */
typedef struct gpl_iter_log {
  int32_t capacity;
  int32_t count;
  float* overflow;           /* [capacity] */
  int64_t* hpwl;             /* [capacity] */
  float* step_length;        /* [capacity] */
  int32_t* backtracks;       /* [capacity] number of tries in the iteration */
} gpl_iter_log;

/* Initial place progress (InitialPlace::doBicgstabPlace). */
typedef struct gpl_ip_stats {
  int32_t iterations;
  float last_error;          /* max(errorX, errorY) of the last round */
  int64_t last_hpwl;         /* PlacerBase::hpwl before the last move */
  int32_t solver_iters_x;    /* BiCGSTAB iterations of the last round */
  int32_t solver_iters_y;
  int32_t cooperative_rounds; /* rounds solved in one launch (cluster or cooperative grid) */
  int32_t pad;
} gpl_ip_stats;

/* Library identity and the last error message of the calling thread. */
const char* gpl_version(void);
const char* gpl_last_error(void);

/* Defaults of replace::Replace::Replace() (src/replace.cpp:13-33) and of the
 * Vars constructors (src/initialPlace.cpp:18-24, src/nesterovBase.cpp:875-880,
 * src/nesterovPlace.cpp:19-29). */
void gpl_params_default(gpl_params* params);

/* Build the job: PlacerBase-level bookkeeping (areas, utilisation check) and
 * the device copy of the netlist.  Replaces `std::make_shared<PlacerBase>(db,
 * log)` in Replace::doInitialPlace / doNesterovPlace (src/replace.cpp:75,96). */
gpl_status gpl_create(const gpl_netlist_desc* netlist, const gpl_params* params,
                      struct gpl_job** job);
void gpl_destroy(struct gpl_job* job);

/* InitialPlace(ipVars, pb, log).doBicgstabPlace() (src/replace.cpp:85-87,
 * src/initialPlace.cpp:56-105): centre the movable instances (unless
 * incremental), then up to initial_place_max_iter B2B + BiCGSTAB rounds. */
gpl_status gpl_initial_place(struct gpl_job* job, gpl_ip_stats* stats);

/* Batched form of gpl_initial_place: the initial places of n_jobs jobs run
 * together (no counterpart in the reference, which places one design per
 * process).  Each job is centred (unless incremental) as gpl_initial_place
 * does; then the B2B + BiCGSTAB rounds of all jobs run in lockstep: each
 * assembly phase and each solver phase is one launch over a table of work
 * items (job, block of that job's own launch, axis), a job leaves when its
 * rounds end (error <= 1e-5 after at least 5 rounds, or
 * initial_place_max_iter).  Every job's result -- instance locations,
 * rounds, error, solver iterations -- is bit-identical to gpl_initial_place
 * on that job alone with the kernel-per-phase solver (ip_solver 0 or 1; the
 * batch always runs that form).  The jobs: distinct, on one device, before
 * gpl_nesterov_init.  stats and status are [n_jobs] (may be NULL): each
 * job's statistics and its gpl_initial_place status; *kernel_launches (may
 * be NULL): kernels launched by the batch.  The call itself returns GPL_OK
 * unless it could not run. */
gpl_status gpl_batch_initial_place(struct gpl_job* const* jobs, int32_t n_jobs, gpl_ip_stats* stats,
                                   gpl_status* status, int64_t* kernel_launches);

/* NesterovBase(nbVars, pb, log) + NesterovPlace::init()
 * (src/replace.cpp:112-125, src/nesterovBase.cpp:917-1062,
 * src/nesterovPlace.cpp:64-175). */
gpl_status gpl_nesterov_init(struct gpl_job* job, gpl_job_info* info);

/* NesterovPlace::doNesterovPlace() (src/nesterovPlace.cpp:275-472), run for
 * at most max_iters further iterations (<= 0: up to nesterov_place_max_iter).
 * Returns GPL_OK while running or converged, or the divergence code. */
gpl_status gpl_nesterov_run(struct gpl_job* job, int32_t max_iters,
                            gpl_nesterov_stats* stats, gpl_iter_log* log);

/* Batched form of gpl_nesterov_run: the Nesterov loops of n_jobs jobs run
 * together (no counterpart in the reference, which places one design per
 * process).  Every round, each running job's next evaluation -- its next
 * back-tracking try or the first try of its next iteration -- joins one
 * persistent launch per phase (scatter, WA, the three Poisson passes, the
 * gcell gradients) driven by a table of work items (job, block of that job's
 * own launch); each job's control then takes its result as gpl_nesterov_run
 * would, and a job leaves the table when its loop ends.  The rounds replay
 * one CUDA graph.  Every job's iterations, log and result are bit-identical
 * to gpl_nesterov_run on that job alone.
 * The jobs: distinct, on one device, after gpl_nesterov_init, on the FFT
 * Poisson form with its shared-memory passes (poisson_path 1, a grid other
 * than 512 x 512 or 1024 x 1024; others return GPL_ERR_INVALID_ARG).
 * max_iters: further iterations per job (<= 0: to the stop rule).  stats and
 * status are [n_jobs] (may be NULL): each job's progress and its
 * gpl_nesterov_run status; *kernel_launches (may be NULL): kernels
 * launched.  The call itself returns GPL_OK unless it could not run. */
gpl_status gpl_batch_nesterov_run(struct gpl_job* const* jobs, int32_t n_jobs, int32_t max_iters,
                                  gpl_nesterov_stats* stats, gpl_status* status, int64_t* kernel_launches);

/* Per-net weights: the hook of GNet::setCustomWeight / GNet::netWeight
 * (src/nesterovBase.h:210-212, src/nesterovBase.cpp:264-266).  The reference
 * stores the weights but does not apply them yet; here each pin's WA gradient
 * (getWireLengthGradientPinWA, src/nesterovBase.cpp:1383-1440) is multiplied
 * by its net's weight before the per-gcell sum (the form timing-driven
 * placers use).  HPWL, the wire-length preconditioner and the initial place
 * stay unweighted.  weights is [n_nets] in the netlist's net order, each
 * finite and >= 0; NULL sets every weight back to 1 (no weighting).  May be
 * called at any time after gpl_create, also between gpl_nesterov_run calls:
 * every later evaluation uses the new weights. */
gpl_status gpl_set_net_weights(struct gpl_job* job, const float* weights, int64_t n_nets);

/* Final locations, NesterovPlace::updateDb (src/nesterovPlace.cpp:585-595):
 * lx = dCx - dDx/2, ly = dCy - dDy/2 for movable instances; other instances
 * keep their input location.  Arrays are [n_insts]. */
gpl_status gpl_get_inst_locations(struct gpl_job* job, int32_t* lx, int32_t* ly);

/* Current Nesterov coordinates (curSLPCoordi_) as float pairs [2 * n_gcells]. */
gpl_status gpl_get_gcell_coords(struct gpl_job* job, float* xy);

/* Gradient check hook: one evaluation at the given gcell centres
 * (updateGCellDensityCenterLocation + updateDensityForceBin +
 * updateWireLengthForceWA + per-gcell getWireLengthGradientWA and
 * getDensityGradient, src/nesterovBase.cpp:1198-1506).  xy, wl_grad and
 * density_grad are [2 * n_gcells]; the two outputs may be NULL. */
gpl_status gpl_eval(struct gpl_job* job, const float* xy, float wl_coef_x,
                    float wl_coef_y, float* wl_grad, float* density_grad,
                    gpl_eval_stats* stats);

/* Bin state after the last evaluation, [bin_cnt_x * bin_cnt_y] row-major by y
 * (bin index j * bin_cnt_x + i, as BinGrid::bins()).  Any pointer may be NULL. */
gpl_status gpl_get_bins(struct gpl_job* job, int64_t* inst_area, int64_t* filler_area,
                        int64_t* non_place_area, float* density, float* phi,
                        float* field_x, float* field_y);

/* Per-gcell density geometry after init: density rectangle [4 * n_gcells]
 * (dLx, dLy, dUx, dUy), density scale [n_gcells], kind [n_gcells]
 * (0 standard cell, 1 macro, 2 filler).  Any pointer may be NULL. */
gpl_status gpl_get_gcells(struct gpl_job* job, int32_t* drect, float* scale, uint8_t* kind);

/* Electrostatic Poisson solve alone (FFT::doFFT, src/fft.cpp:112-177) on
 * device arrays: density, phi, field_x and field_y are device pointers of
 * [ny * nx] floats, row-major by y.  nx, ny: powers of two in [2, 4096].
 * Scratch memory is allocated on first use per device and grid and cached
 * for the device's current context (after cudaDeviceReset the entries of
 * the old context are dropped, not freed, and new scratch is allocated).
 * stream: cudaStream_t (NULL = default stream). */
gpl_status gpl_poisson_solve(int32_t nx, int32_t ny, int32_t bin_size_x,
                             int32_t bin_size_y, const float* density, float* phi,
                             float* field_x, float* field_y, void* stream);

/* Allocation-free variant of gpl_poisson_solve.  It has no counterpart in
 * the reference.  It serves callers that must not allocate device memory
 * during the call (a server that admits jobs against a fixed HBM budget, a
 * framework whose caching allocator owns the device memory, a loop that
 * cannot absorb cudaMalloc/cudaFree synchronisation): its scratch is a fixed
 * static device array (about 3.1 MB, held by every GPU that loads the
 * library) and the call allocates nothing.  Limit: nx * ny <= 512 * 512
 * (larger grids return GPL_ERR_INVALID_ARG).  The first call on a device
 * looks up the array's device address; make that first call before any
 * stream capture.  The address is kept per device context: the first call
 * after a cudaDeviceReset looks it up again (also before any capture).  All
 * calls share the array, so calls that overlap on the GPU race; order them
 * (same stream, or events). */
gpl_status gpl_poisson_solve_noalloc(int32_t nx, int32_t ny, int32_t bin_size_x,
                                     int32_t bin_size_y, const float* density, float* phi,
                                     float* field_x, float* field_y, void* stream);

/* Kernel timing hook used by the benchmark: accumulates CUDA-event time of
 * the job's kernels by class since the last reset.  names/ms/launches are
 * [capacity]; returns the number of classes written. */
int32_t gpl_kernel_times(struct gpl_job* job, const char** names, double* ms,
                         int64_t* launches, int32_t capacity);
void gpl_kernel_times_reset(struct gpl_job* job, int32_t enable);
/* Number of kernels the job has launched since the last reset. */
int64_t gpl_kernel_launch_count(struct gpl_job* job);

/* Tensor-core GEMM (no reference counterpart; the building block of the
 * DCT-as-GEMM Poisson path): D (m x n, fp32, row-major) = A (m x k, bf16,
 * row-major) * B (n x k, bf16, row-major)^T on tcgen05 with TMA-fed shared
 * memory.  All pointers are device memory, 16-byte aligned; m must be a
 * multiple of 128, n and k of 64.  *error_flag (device int, may be NULL) is
 * set to 1 if a pipeline wait timed out (the result is then invalid). */
gpl_status gpl_tc_gemm_bf16(const void* a, const void* b, float* d, int32_t m, int32_t n, int32_t k,
                            int32_t* error_flag, void* stream);

/* ------------------------------------------------------------------------
 * Placement server: continuous batching of independent jobs on one GPU.
 * No reference counterpart: RePlAce places one design per process.  A
 * server keeps up to max_active jobs resident and running at once, each on
 * its own stream with its own CUDA graph, so their kernels overlap on the
 * device.  Jobs are admitted in submission order as a slot frees and their
 * device footprint (an upper bound, computed at submission) fits the HBM
 * budget next to the jobs already resident; a job joins when admitted and
 * retires when its Nesterov loop ends, between iterations.  Each job runs
 * the same kernels on its own buffers as gpl_create + gpl_initial_place +
 * gpl_nesterov_init + gpl_nesterov_run would, so its result does not depend
 * on the other jobs.
 * Threading: the server's calls may come from any thread; it runs one host
 * thread per slot. */
typedef struct gpl_server gpl_server;

typedef struct gpl_server_params {
  int32_t device;             /* CUDA device ordinal */
  int32_t max_active;         /* slots: jobs resident and running at once (8) */
  int64_t hbm_budget_bytes;   /* device bytes the jobs may hold together;
                                 0 = 80 % of the free memory at creation */
  int32_t chunk_iters;        /* Nesterov iterations between cancel checks (64) */
  int32_t run_initial_place;  /* 1 = gpl_initial_place before the Nesterov loop (1) */
  int32_t blocking_sync;      /* 1 = slot threads sleep while waiting for the GPU (1) */
  int32_t batched;            /* 1 = admitted jobs run their Nesterov loops together as
                                 one batch (gpl_batch_nesterov_run's kernels): a job joins
                                 the running batch when its initialisation is done and
                                 leaves it when its loop ends; jobs the batched kernels do
                                 not cover (512 x 512 and 1024 x 1024 grids) run alone on
                                 their slot.  Jobs with poisson_path 0 (auto) take the FFT
                                 form (1) in this mode.  0 = every job runs its own loop
                                 on its slot's stream (0) */
} gpl_server_params;

typedef struct gpl_server_result {
  int64_t ticket;
  int32_t status;             /* gpl_status of the job */
  int32_t finished;           /* 1 = the Nesterov loop reached its stop rule */
  int32_t iterations;         /* Nesterov iterations */
  int32_t ip_rounds;          /* initial-place rounds */
  float overflow;             /* final overflow */
  int32_t n_insts;
  int64_t hpwl;               /* final pin HPWL (DBU) */
  int64_t device_bytes;       /* footprint reserved at admission */
  double submit_s, admit_s, finish_s;   /* seconds since the server started */
  char message[160];          /* gpl_last_error text when status != 0 */
} gpl_server_result;

void gpl_server_params_default(gpl_server_params* p);
gpl_status gpl_server_create(const gpl_server_params* p, gpl_server** out);
/* Copies the netlist (the caller's arrays may be freed on return) and queues
 * the job.  Invalid netlists and jobs whose footprint exceeds the budget are
 * rejected here.  *ticket identifies the job in the calls below. */
gpl_status gpl_server_submit(gpl_server* s, const gpl_netlist_desc* nl, const gpl_params* p,
                             int64_t* ticket);
/* gpl_server_submit with per-net weights (as gpl_set_net_weights; weights
 * [n_nets] are copied, NULL means unweighted). */
gpl_status gpl_server_submit_weighted(gpl_server* s, const gpl_netlist_desc* nl, const gpl_params* p,
                                      const float* weights, int64_t n_nets, int64_t* ticket);
/* Up to capacity results of jobs that ended since the last poll, waiting up
 * to wait_ms for the first one; returns how many were written. */
int32_t gpl_server_poll(gpl_server* s, gpl_server_result* out, int32_t capacity, int32_t wait_ms);
/* Final instance locations of an ended job ([n_insts] each), as
 * gpl_get_inst_locations gives them. */
gpl_status gpl_server_get_inst_locations(gpl_server* s, int64_t ticket, int32_t* lx, int32_t* ly);
/* Drops an ended job's result and locations. */
gpl_status gpl_server_release(gpl_server* s, int64_t ticket);
/* A queued job ends at once; a running one at its next chunk boundary. */
gpl_status gpl_server_cancel(gpl_server* s, int64_t ticket);
/* Numbers of jobs queued, running and ended-but-not-polled. */
void gpl_server_counts(gpl_server* s, int32_t* queued, int32_t* running, int32_t* ended);
/* Cancels queued jobs, waits for the running ones, frees everything. */
void gpl_server_destroy(gpl_server* s);

#ifdef __cplusplus
}
#endif

#endif /* GPL_GB300_GPL_H */
