/*
 * sg_solver.h -- C ABI of the GB300 solve path for SPECFEM3D_GEOTECH.
 *
 * Every entry point is plain C: integers, doubles and pointers to host
 * arrays, no CUDA or torch types.  Each call returns an errcode (SG_OK = 0)
 * and, where the reference has one, fills a blank-padded Fortran-style
 * errtag of SG_ERRTAG_LEN characters.  Array layouts follow the reference:
 *   - global vectors are 0:neq (length neq+1); index 0 is the sink of the
 *     constrained dofs and holds 0;
 *   - element matrices k(nedof,nedof,nelmt) are column-major, element e's
 *     81x81 block is 6561 consecutive doubles, k[(e*81 + col)*81 + row];
 *   - gdof_elmt(nedof,nelmt): gdof_elmt[e*81 + a] in [0,neq], 0 = fixed,
 *     dofs node-major inside an element [n1x n1y n1z n2x ...];
 *   - hex8 connectivity is 1-based in Exodus/CUBIT corner order, material ids
 *     are 1-based, face ids 1..6 follow src/element.f90:48-141.
 * A context (sg_ctx) owns the device, a stream and all device memory; one
 * context is used by one host thread at a time.
 */
#ifndef SG_SOLVER_H
#define SG_SOLVER_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SG_ERRTAG_LEN 250

enum sg_status {
  SG_OK = 0,
  SG_ERR_NOCONV = -1,   /* PCG did not converge: same code as the reference's errcode -1 */
  SG_ERR_TIMEOUT = -2,  /* a device loop hit its wall-clock or iteration guard */
  SG_ERR_OOM = -3,      /* the request does not fit the context's HBM budget */
  SG_ERR_BADARG = -4,   /* invalid sizes, indices or options */
  SG_ERR_CUDA = -5,     /* a CUDA runtime error; see sg_last_error */
  SG_ERR_NODEVICE = -6  /* no CUDA device / the kernels are not loadable */
};

/* Precision forms of the device-resident solve. */
enum sg_precision {
  SG_PREC_FP64 = 0,   /* plain: FP64 element matrices, FP64 PCG (the drop-in semantics) */
  SG_PREC_MIXED = 1   /* FP32 element matrices and FP32 PCG, FP64 iterative refinement */
};

typedef struct sg_ctx sg_ctx;
typedef struct sg_model sg_model;
typedef struct sg_mesh sg_mesh;

/* ---- context ---------------------------------------------------------- */
/* Creates a context on CUDA device `device`.  hbm_budget = 0 means all free
 * device memory.  Returns NULL if no device is usable (sg_create_status tells why). */
sg_ctx* sg_create(int device, size_t hbm_budget);
int sg_create_status(void);
void sg_destroy(sg_ctx* ctx);
const char* sg_last_error(const sg_ctx* ctx);
/* Device memory currently held by the context, bytes. */
size_t sg_hbm_used(const sg_ctx* ctx);

/* ---- the plain drop-in: pcg_solver ------------------------------------ */
/* Replaces subroutine pcg_solver(neq,nelmt,k,u,f,dprecon,gdof_elmt,cg_iter,
 * errcode,errtag) of module solver (src/solver.f90:14-79); the module globals
 * cg_maxiter, cg_tol and nedof (src/solver.f90:8) are passed explicitly.
 * Diagonally preconditioned CG on the element-by-element operator, warm start
 * from u when max|u| > 0, stop when |alpha|*max|p|/max|u| <= cg_tol.  Only u
 * is modified.  Returns SG_OK (cg_iter = stopping iteration) or
 * SG_ERR_NOCONV with errtag "ERROR: PCG solver doesn't converge!". */
int sg_pcg_solve(sg_ctx* ctx, int neq, int nelmt, int nedof, const double* k, double* u,
                 const double* f, const double* dprecon, const int* gdof_elmt, int cg_maxiter,
                 double cg_tol, int* cg_iter, char* errtag);

/* Replaces the stress / yield / viscoplastic-flow / body-load block that the
 * plastic loops inline after each pcg_solver call: src/slope.F90:311-383, and
 * its excavation copy src/excavation.F90:546-616.  With sg_pcg_solve it lets a
 * host keep its own plastic loop and run both heavy steps on the GPU.  Arrays
 * are the reference's own, ids 1-based:
 *   g_coord[3*nnode], g_num[27*nelmt] (nodes 1..nnode, GLL order i+3j+9k),
 *   gdof_elmt[81*nelmt] in [0,neq], mat_id[nelmt] in [1,nmatblk];
 *   ym_blk and the factored nuf/phif/cohf/psif_blk[nmatblk] (angles in degrees,
 *   src/plastic_library.f90:42-88), dt (src/plastic_library.f90:17-39);
 *   elmt_list[nel]: elements 1..nelmt to visit in order (elmt_intact), or NULL
 *   for all nelmt;
 *   x[neq+1]; evpt and stress_elmt[6*27*nelmt] in/out;
 *   bodyload[neq+1] in/out: the element loads are added in element order
 *   unless last, and bodyload[0] is set to 0;
 *   wpressure[nnode] or NULL: pore pressure added to the normal effective
 *   stress (0 on nodes that are not submerged);
 *   form 0: slope order (pressure after the stored stress);
 *   form 1: excavation order (pressure before it), and when last, vmeps[nnode]
 *   += the points' von Mises plastic strain and scf[nnode] = min(scf, point
 *   safety factor) (either may be NULL);
 *   last = nl_isconv .or. nl_iter == nl_maxiter: the stress is stored, no load.
 * fmax receives max(0, max F) over the visited points.  The mesh, dof map,
 * material ids and element list are uploaded only when they change between
 * calls; the plastic state is copied in and out on every call. */
int sg_stress_bodyload(sg_ctx* ctx, int neq, int nelmt, int nnode, const double* g_coord, const int* g_num,
                       const int* gdof_elmt, const int* mat_id, int nmatblk, const double* ym_blk,
                       const double* nuf_blk, const double* phif_blk, const double* cohf_blk,
                       const double* psif_blk, double dt, int nl_isconv, int last, const int* elmt_list,
                       int nel, const double* wpressure, int form, const double* x, double* evpt,
                       double* stress_elmt, double* bodyload, double* vmeps, double* scf, double* fmax,
                       char* errtag);

/* No counterpart in the reference.  The same solve as sg_pcg_solve (same
 * arguments and results, host arrays in and out) for callers that cannot
 * allocate device memory -- code that runs under its own memory pool or
 * sub-allocator, or that must not call cudaMalloc at all.  It needs no
 * context: all device memory it uses is one static device array of 64 MiB
 * held by every GPU that loads the library until the process exits, and it
 * calls no cudaMalloc, cudaFree or other allocating routine.  Problems whose
 * arrays need more than 64 MiB are rejected with SG_ERR_BADARG (the dense
 * 81x81 FP64 element matrices alone take 52.5 KB per element, so about
 * 1,100 elements fit).  The first call on a device looks up the array's
 * device address; make it before any stream capture.  Calls share the
 * array: each call clears what must start at zero, and calls that overlap on
 * the GPU race and must be serialised by the caller.  Runs on the current
 * device, on the legacy default stream, and returns when done. */
int sg_pcg_solve_noalloc(int neq, int nelmt, int nedof, const double* k, double* u, const double* f,
                         const double* dprecon, const int* gdof_elmt, int cg_maxiter, double cg_tol,
                         int* cg_iter, char* errtag);

/* ---- host-only mesh (no device) ---------------------------------------- */
/* Reads a .sem deck -- or a .psem deck, whose nproc, part_path and gfile
 * entries are ignored and whose unpartitioned input files are read -- and
 * builds the 27-node mesh, face constraints and node-major dof numbering on the
 * host: read_input (src/read_input.f90:13-619), hex2spec (src/mesh_spec.f90:17-386)
 * and apply_bc (src/apply_bc.f90:7-143), the same code sg_model_from_deck runs
 * before it uploads.  Needs no GPU.  NULL with errtag (the reference's message
 * where it has one) on failure. */
sg_mesh* sg_mesh_from_deck(const char* sem_path, char* errtag);
void sg_mesh_free(sg_mesh* mesh);
/* info[0..7] = nnode, nelmt, neq, nmatblk, nsrf, nexcav, iswater, nwmat */
int sg_mesh_info(const sg_mesh* mesh, int* info);
/* g_coord[3*nnode], g_num[27*nelmt] (0-based), gdof[3*nnode], gdof_elmt[81*nelmt],
 * mat_id[nelmt] (1-based), props[6*nmatblk] (gamma E nu phi c psi); any may be NULL. */
int sg_mesh_arrays(const sg_mesh* mesh, double* g_coord, int* g_num, int* gdof, int* gdof_elmt, int* mat_id,
                   double* props);
/* dctl[8] = cg_tol, nl_tol, z0, s0, k0, eqkx, eqky, eqkz;
 * ictl[8] = cg_maxiter, nl_maxiter, phinu, allelastic, nexcav, ninc, s0_type (-1: no
 * stress0 line), iseqload; srf[nsrf]; nexcavid[nexcav] and excavid[sum of nexcavid];
 * water_ids[nwmat]; any may be NULL. */
int sg_mesh_control(const sg_mesh* mesh, double* dctl, int* ictl, double* srf, int* nexcavid, int* excavid,
                    int* water_ids);

/* ---- device-resident model -------------------------------------------- */
/* Builds a spectral (27-node) model from an 8-node hex mesh: hex2spec with
 * node merging (src/mesh_spec.f90:17-386), face constraints and node-major dof
 * numbering (src/apply_bc.f90:7-143), then uploads the mesh and builds the
 * element matrices, diagonal preconditioner and gravity load on the device
 * (src/preprocess.f90:74-148).
 *   props: nmatblk rows of [gamma E nu phi c psi] (src/read_input.f90:563-595)
 *   bc_counts[3]: number of (element,face) pairs fixing ux, uy, uz
 *   bc_pairs: the pairs, ux list then uy then uz, 2 ints each
 *   precision: SG_PREC_FP64 or SG_PREC_MIXED (which element-matrix copies to keep) */
sg_model* sg_model_from_hex8(sg_ctx* ctx, int nnode8, const double* x8, const double* y8,
                             const double* z8, int nelmt, const int* conn8, const int* mat_id,
                             int nmatblk, const double* props, const int* bc_counts,
                             const int* bc_pairs, int precision, char* errtag);
/* Reads a serial .sem deck (preinfo/mesh/bc/material/control/stress0/eqload/water
 * lines, src/read_input.f90:13-619) and builds the model as above; a water: line
 * sets the model's pore pressure as sg_model_set_water does. */
sg_model* sg_model_from_deck(sg_ctx* ctx, const char* sem_path, int precision, char* errtag);
void sg_model_free(sg_model* model);
/* info[0..7] = nnode, nelmt, neq, nmatblk, nsrf (deck), ngroups, 0, 0 */
int sg_model_info(const sg_model* model, int* info);
/* Host copies of the spectral mesh (any pointer may be NULL):
 * g_coord[3*nnode], g_num[27*nelmt] (0-based nodes), gdof[3*nnode], gdof_elmt[81*nelmt]. */
int sg_model_arrays(const sg_model* model, double* g_coord, int* g_num, int* gdof, int* gdof_elmt);
/* Deck control values: dctl = {cg_tol, nl_tol}, ictl = {cg_maxiter, nl_maxiter, phinu,
 * allelastic, nexcav, ninc}, srf (nsrf doubles, may be NULL). */
int sg_model_control(const sg_model* model, double* dctl, int* ictl, double* srf);
/* Element matrices (column-major 81x81 per element, FP64), diagonal
 * dprecon (0:neq, before inversion) and gravity load extload (0:neq) as built on
 * the device by stiffness_bodyload; any pointer may be NULL. */
int sg_model_stiffness(sg_model* model, double* storekm, double* dprecon, double* extload);
/* Pseudo-static earthquake load (the deck's eqload: line, src/read_input.f90:293-303,
 * applied as in src/preprocess.f90:137-143): every later slope trial's external
 * load gains eqk * gamma * w detJ per node and direction on top of gravity.  The
 * excavation driver keeps gravity alone (src/excavation.F90:191).  Rebuilds the
 * stiffness and loads; SG_ERR_BADARG while a trial batch is open. */
int sg_model_set_eqload(sg_model* model, double eqkx, double eqky, double eqkz);
/* Water table (the deck's water: line and the material list's water IDs,
 * src/read_input.f90:307-317,602-611; compute_pressure, src/compute_pressure.f90:10-186,
 * replaced on the device): nodes of elements whose material is one of water_ids
 * (1-based, nwmat of them) are submerged, and a submerged node under the first
 * surface of wsfile that covers it gets the pore pressure 9.81 (z_surface - z).
 * Every later slope trial and excavation stage adds that pressure to the normal
 * components of the effective stress at the node's GLL points (src/slope.F90:334-341,
 * src/excavation.F90:566-576).  Errors: the file cannot be read, a water ID out of
 * range, a meshed surface whose z cannot be determined ("ERROR: free surface cannot
 * be determined!") -> SG_ERR_BADARG with errtag; SG_ERR_BADARG while a trial batch is open. */
int sg_model_set_water(sg_model* model, const char* wsfile, const int* water_ids, int nwmat, char* errtag);
/* Sets the pore pressure directly (nnode values, node order of sg_model_arrays;
 * 0 on nodes that are not submerged); NULL removes it. */
int sg_model_set_pore_pressure(sg_model* model, const double* wpressure);
/* Reads the pore pressure back (nnode values); SG_ERR_BADARG when none is set. */
int sg_model_pore_pressure(const sg_model* model, double* wpressure);

/* ---- one strength-reduction trial of slope3d (src/slope.F90:244-443) ---- */
typedef struct sg_control {
  double cg_tol;       /* PCG step tolerance (reference cg_tol) */
  double nl_tol;       /* plastic-iteration tolerance (reference nl_tol) */
  int cg_maxiter;
  int nl_maxiter;
  int phinu;           /* phi-nu correction of strength_reduction */
  int allelastic;
  int precision;       /* sg_precision */
  int reserved;
  double refine_rtol;  /* SG_PREC_MIXED: FP64 relative residual target (default 1e-10) */
  double inner_rtol;   /* SG_PREC_MIXED: FP32 residual reduction between FP64 residual replacements (default 1e-3) */
} sg_control;

typedef struct sg_trial_result {
  double srf;
  int cg_tot;          /* summed PCG iterations (summary column CGITER) */
  int nl_iter;         /* plastic iterations (summary column NLITER) */
  int converged;       /* nl_isconv at exit */
  int failed;          /* nl_iter == nl_maxiter: the SRF loop's exit test */
  double uxmax, umax, fmax, uerr;
  int errcode;         /* SG_OK or the PCG error */
  int refine_steps;    /* SG_PREC_MIXED: FP64 residual evaluations */
  double seconds;      /* device wall time of the trial */
} sg_trial_result;

/* Runs k independent SRF trials of the model's mesh concurrently (k = 1 is
 * the plain one-at-a-time slope3d trial).  Trials share the element matrices
 * and are batched as k right-hand sides of the element apply; each keeps its
 * own factored properties, plastic strain, stress, body load and iteration
 * counts.  Valid only when the stiffness does not depend on the SRF
 * (phinu = 0 or no phi-nu correction triggered); otherwise returns SG_ERR_BADARG.
 * x_out (optional, k*(neq+1)) receives each trial's displacement. */
int sg_srf_trials(sg_model* model, const sg_control* ctl, int k, const double* srf,
                  sg_trial_result* results, double* x_out);

/* ---- continuous batching of SRF trials on one model -------------------
 * A batch has kmax (<= 16) slots.  sg_batch_add starts a trial in a free
 * slot at any time, sg_batch_step advances every running trial by up to
 * nsteps plastic iterations (one shared multi-RHS solve per iteration),
 * sg_batch_poll reports a slot (state 0 free, 1 running, 2 finished) and
 * sg_batch_release frees a finished slot for the next trial.  sg_srf_trials
 * is begin + add + step-to-completion + end. */
int sg_batch_begin(sg_model* model, const sg_control* ctl, int kmax);
int sg_batch_add(sg_model* model, double srf, int* slot);
int sg_batch_step(sg_model* model, int nsteps, int* nlive);
int sg_batch_poll(sg_model* model, int slot, sg_trial_result* result, int* state);
int sg_batch_release(sg_model* model, int slot);
int sg_batch_end(sg_model* model);

/* Stress state of the last trial batch: stress[(t*nelmt + e)*27*6 + i*6 + s] for trial t. */
int sg_last_stress(sg_model* model, int trial, double* stress_elmt);
/* Valency-averaged nodal stress of trial t of the last batch, stress_global[n*6 + s]
 * (src/slope.F90:419-437: element stresses summed per node in element order, divided
 * by the node's valency), reduced on the device. */
int sg_nodal_stress(sg_model* model, int trial, double* stress_global);

/* ---- outputs (host only; no device needed) ----------------------------- */
/* Per node (src/postprocess.f90:146-183): principal stresses psigma[3n..3n+2] in
 * ascending order (compression first), maximum shear stress taumax[n] = |p1 - p3|/2 and
 * normal stress on its plane nsigma[n] = (p1 + p3)/2 (taumax, nsigma may be NULL). */
int sg_principal_stress(int nnode, const double* stress_global, double* psigma, double* taumax, double* nsigma);
/* Summary file (src/semgeotech.F90:315-319, src/slope.F90:213-220): banner, control
 * values and the column header; then one row per SRF trial (src/slope.F90:409-416):
 * srf cg_tot nl_iter uxmax umax fmax. */
int sg_write_summary_header(const char* path, const sg_control* ctl, int nsrf);
int sg_write_summary_row(const char* path, const sg_trial_result* result);
/* EnSight Gold C-binary output (src/semgeotech.F90:126-312, src/visual.f90):
 * the .case file of a slope run (displacement vector and symmetric stress tensor per
 * node, one time value per SRF step, files <head>_step<NNN>.dis/.sig), the geometry
 * (every 27-node element as 8 hexa8 cells, Exodus corner order; g_num 0-based) and one
 * per-node variable (ncomp 1, 3 or 6; var[n*ncomp + c]). */
int sg_write_ensight_case(const char* path, const char* head, int nsteps, const double* times, int tstart);
int sg_write_ensight_geo(const char* path, int nnode, const double* g_coord, int nelmt, const int* g_num);
int sg_write_ensight_var(const char* path, const char* description, int ncomp, int nnode, const double* var);

/* The slope3d SRF sweep: trials srf[0..nsrf) in order, stopping after the first
 * failed trial (src/slope.F90:441).  Returns the number of trials run in *ndone. */
int sg_srf_sweep(sg_model* model, const sg_control* ctl, int nsrf, const double* srf,
                 sg_trial_result* results, int* ndone);

/* Critical SRF on the grid lo + step*m (m = 0..round((hi-lo)/step)) by
 * bisection, assuming lo is stable and hi fails (the failure test of the
 * reference's SRF loop: nl_iter == nl_maxiter, src/slope.F90:441).  k = 1
 * runs the bisection one trial at a time.  k > 1 runs the same bisection with
 * its next probes ahead in a batch of k trials: free slots take the
 * shallowest undecided probes of the current node's subtree, results are
 * applied in the bisection's own order and probes in the subtree not taken
 * are cancelled, so the answer is the bisection's for any pattern of
 * failures.  *ntrials = trials started; *nrounds = bisection steps (k = 1) or
 * result events waited for (k > 1).  The environment variable
 * SG_FOS_SEARCH=ksection selects a k-section instead (each result moves the
 * bracket; the bisection's answer only where failure is monotone in SRF). */
int sg_fos(sg_model* model, const sg_control* ctl, double lo, double hi, double step, int k,
           double* fos, int* ntrials, int* nrounds);
/* Plastic iterations run by the model's last sg_fos: batch iterations for
 * k > 1 (one iteration of all the batch's trials counts once), trial
 * iterations summed over the bisection's trials for k = 1.  No counterpart in
 * the reference (its SRF loop prints per-trial counts only). */
int sg_fos_steps(const sg_model* model, long long* steps);

/* ---- request loop: factor-of-safety and excavation solves of many meshes --
 * Requests are queued on submission and admitted in arrival order when their
 * estimated HBM footprint fits the server's budget (hbm_budget = 0: 90 % of
 * free device memory).  `workers` threads each own a context and stream, so
 * admitted requests run concurrently on the device; inside a factor-of-safety
 * request the SRF search is sg_fos with k batched trials, an excavation
 * request runs sg_excavation.  Times are seconds since the server was created. */
typedef struct sg_server sg_server;
typedef struct sg_fos_result {
  int id, status;
  double fos;
  int ntrials, nrounds, nelmt, neq;
  double footprint, hbm_bytes;        /* admission estimate, device bytes used */
  double t_arrival, t_start, t_done;
  int kind;    /* 0 factor of safety; 1 staged excavation (fos unused, ntrials = plastic
                  iterations over the stages run, rows from sg_server_stages) */
  int nstage;  /* excavation: stages run */
} sg_fos_result;
sg_server* sg_server_create(int device, size_t hbm_budget, int workers);
int sg_server_submit(sg_server* server, int nnode8, const double* x8, const double* y8, const double* z8,
                     int nelmt, const int* conn8, const int* mat_id, int nmatblk, const double* props,
                     const int* bc_counts, const int* bc_pairs, const sg_control* ctl, double lo,
                     double hi, double step, int k, int* id);
/* Queues a staged-excavation request (sg_excavation on its own model; the
 * stage arguments as there), admitted by its footprint like the others. */
int sg_server_submit_excavation(sg_server* server, int nnode8, const double* x8, const double* y8,
                                const double* z8, int nelmt, const int* conn8, const int* mat_id, int nmatblk,
                                const double* props, const int* bc_counts, const int* bc_pairs,
                                const sg_control* ctl, int s0_type, double z0, double s0, double k0, int nexcav,
                                const int* nexcavid, const int* excavid, int ninc, double srf, int* id);
/* The stage rows of a finished excavation request (nstage rows of 8, as sg_excavation). */
int sg_server_stages(sg_server* server, int id, double* stage_res);
/* Blocks until request `id` is done (or timeout_s passes: SG_ERR_TIMEOUT). */
int sg_server_wait(sg_server* server, int id, double timeout_s, sg_fos_result* result);
/* stats[0..5] = completed, p50 latency, p99 latency (arrival to done, s),
 * completed / (last done - first arrival), peak concurrent requests, budget bytes. */
int sg_server_stats(sg_server* server, double* stats);
void sg_server_destroy(sg_server* server);

/* ---- staged excavation (src/excavation.F90:15-709), nsrf = 1 ---------- */
/* s0_type 1: overburden initial stress s0 - gamma*|z - z0| with K0
 * (src/postprocess.f90:10-33); s0_type 0: elastic gravity solve
 * (src/excavation.F90:182-238).  nexcavid[i] ids per stage, excavid the ids.
 * stage_res: nexcav rows of [stage cg_tot nl_tot uxmax umax fmax failed errcode].
 * Returns the number of stages run in *nstage. */
int sg_excavation(sg_model* model, const sg_control* ctl, int s0_type, double z0, double s0,
                  double k0, int nexcav, const int* nexcavid, const int* excavid, int ninc,
                  double srf, double* stage_res, int* nstage);
/* Nodal fields of the last completed excavation stage (src/excavation.F90:597-661):
 * vmeps[n], the von Mises effective plastic strain sqrt(2/3 evpt.evpt) summed over the
 * intact elements at node n and divided by its intact valency, and scf[n], the smallest
 * safety factor (sigm sin(phi) - c cos(phi)) / (-dsbar (cos(theta)/sqrt(3) -
 * sin(theta) sin(phi)/3)) of those points (1e32 where none).  Either may be NULL. */
int sg_excavation_fields(const sg_model* model, double* vmeps, double* scf);

/* ---- timing of the device work of the last call ----------------------- */
/* ms[0] total, ms[1] element apply, ms[2] gather, ms[3] PCG vector update,
 * ms[4] stress update, ms[5] stiffness build; counts[0..3] = launches of the
 * apply kernel, total kernel launches, PCG iterations, FP64 refinement residuals.
 * Collected with CUDA events on the context's stream when enabled. */
int sg_profile_enable(sg_ctx* ctx, int on);
int sg_profile_read(sg_ctx* ctx, double* ms, long long* counts);
/* CUDA-event marks on the context's stream (id 0..15) and the device time
 * between two marks in milliseconds (synchronises on mark b). */
int sg_timer_mark(sg_ctx* ctx, int id);
double sg_timer_ms(sg_ctx* ctx, int a, int b);

#ifdef __cplusplus
}
#endif
#endif /* SG_SOLVER_H */
