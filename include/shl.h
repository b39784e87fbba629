/*
 * shl.h -- C ABI of the GB300 shell library (libshl_gb300.so).
 *
 * The library is a drop-in for the per-step force evaluation and explicit
 * Newmark integration of the Loop-subdivision Koiter shell solver
 * (ShellSystem::advance and everything it calls, ShellSystem.C:952-1122).
 * A host driver keeps the mesh, the config.cfg parameters and the state file,
 * and calls these entry points from its time loop in place of
 * `system.advance(time_step)` (shell.C:340).
 *
 * Conventions
 *  - Plain C types only.  Host arrays are owned by the caller and copied.
 *  - Node-major vectors: x[3*nid + c], c = 0,1,2; node and face ids are the
 *    order of the OFF file (0-based).
 *  - Every call returns a shl_status; nothing throws or exits.  Values 1..7
 *    equal ShellSystem::Problem (ShellSystem.h:48-49); values >= 100 are
 *    errors of the library itself.
 *  - A context owns its device memory and one CUDA stream; it is not
 *    thread-safe (one host thread per context).
 *  - All arithmetic is FP64 unless a precision mode says otherwise.
 */
#ifndef SHL_H_
#define SHL_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ShellSystem::Problem (ShellSystem.h:48-49) + library errors. */
typedef enum shl_status {
  SHL_OK = 0,
  SHL_NO_DISP_CHANGE = 1,
  SHL_LARGE_DISP = 2,
  SHL_STOP_SIM = 3,
  SHL_TOO_MANY_CELLS = 4,
  SHL_SMALL_TIMESTEP = 5,
  SHL_CONTACT_PROBLEM = 6,
  SHL_NOT_FINITE = 7,
  SHL_ERR_ARG = 100,     /* invalid argument or unsupported option */
  SHL_ERR_CUDA = 101,    /* a CUDA call failed; see shl_last_error() */
  SHL_ERR_TIMEOUT = 102, /* a bounded device wait ran out */
  SHL_ERR_OOM = 103,     /* device allocation failed */
  SHL_ERR_CAPACITY = 104 /* a device buffer (e.g. contact pairs) is too small */
} shl_status;

/* ShellSystem::ContactType (ShellSystem.h:46).  LINEAR: closest points of the
 * flat triangles (ShellShellContact.C); SMOOTH: closest points of the Loop
 * limit surfaces of the two faces, searched from the pair's previous solution
 * (SmoothShellShellContact.C); both distribute the contact force linearly over
 * the faces' nodes (ShellSystem.C:1862-1890). */
enum { SHL_CONTACT_LINEAR = 0, SHL_CONTACT_SMOOTH = 1, SHL_CONTACT_NONE = 2 };
/* ShellSystem::CoordinateSystem (ShellSystem.h:42) for pressure_base. */
enum { SHL_CS_LOCAL = 0, SHL_CS_CARTESIAN = 1, SHL_CS_CYLINDRICAL = 2, SHL_CS_SPHERICAL = 3 };
/* Element-force precision. */
enum { SHL_PREC_FP64 = 0, SHL_PREC_FP32 = 1 };

/* A closed triangle mesh (the OFF file after refinement/projection,
 * shell.C:147-230).  Faces are outward oriented. */
typedef struct shl_mesh {
  uint32_t n_nodes;
  uint32_t n_faces;
  const double* xyz;      /* 3*n_nodes */
  const uint32_t* faces;  /* 3*n_faces */
} shl_mesh;

/* The parameters of ShellSystem::set_parameters (ShellSystem.C:170-418) that
 * act on the time step.  Names follow config.cfg. */
typedef struct shl_params {
  /* material (ShellSystem.C:176-186) */
  double shell_mass_density;
  double shell_young_modulus;   /* E1 */
  double shell_young_modulus2;  /* E2 */
  double shell_poisson_ratio;   /* nu12 */
  double shell_shear_modulus;   /* G12 */
  double bulk_modulus;
  double memb_stiff_mult;
  double bend_stiff_mult;
  double thickness;
  /* dynamics (ShellSystem.C:215-233) */
  double damping_alpha;
  double damping_beta;
  double damping_gamma;
  double pressure;        /* used when a step gets no per-step pressure table */
  int32_t pressure_base;  /* SHL_CS_* */
  int32_t pressure_dir;   /* 0,1,2 */
  /* self-contact (ShellSystem.C:256-276) */
  int32_t shell_shell_contact;  /* SHL_CONTACT_* */
  int32_t pad0;
  double mu_s, mu_d;
  double self_damping;
  double self_friction_damping;
  double fric_stiff_mult;
  double friction_stop_velocity;
  double static_friction_tol;
  double cell_size_mult;
  double cell_margin;
  double neighbor_margin;
  /* time integration (ShellSystem.C:285-313) */
  double dt;
  double newmark_beta;
  double newmark_gamma;
  /* reproduce ShellSystem.C:1480, where the pressure is multiplied by a
   * global that is never assigned (so it is always zero) */
  int32_t compat_zero_pressure;
  /* element-force precision, SHL_PREC_* */
  int32_t precision;
  /* stop after any problem, not only after those >= SHL_STOP_SIM
   * (ShellSystem.C:289, 2952) */
  int32_t stop_on_problem;
  int32_t pad1;
  /* adaptive time stepping (ShellSystem.C:291-313, 1010-1044, 1104-1117):
   * every adapt_dt_every-th step estimates the local error and retries the
   * step with a smaller dt when it is too large; 0 = fixed dt */
  uint32_t adapt_dt_every;
  int32_t pad2;
  double dt_min;            /* 0 = machine epsilon */
  double dt_max;            /* 0 = unbounded */
  double rel_loc_err_min;
  double rel_loc_err_max;
  /* cavity contact (ShellSystem.C:1600-1723): the shell is kept inside a box,
   * a cylinder (axis x) or an ellipsoid of semi-axes Rx, Ry, Rz, with linear
   * penalty contact, normal damping and Coulomb friction per node */
  int32_t shell_cavity_contact;
  int32_t cavity;         /* SHL_CAVITY_* */
  double Rx, Ry, Rz;      /* constant semi-axes; see shl_set_cavity_functions */
  double mu_s_cavity, mu_d_cavity;
  double cavity_damping;
  double cavity_friction_damping;
} shl_params;

/* ShellSystem::CavityType (ShellSystem.h:44). */
enum { SHL_CAVITY_BOX = 0, SHL_CAVITY_CYLINDER = 1, SHL_CAVITY_ELLIPSOID = 2 };

/* Scalars measured in a step (ShellSystem.C:2686-2846). */
typedef struct shl_energies {
  double Etens, Ebend;    /* elastic energies at the predicted state */
  double Eself, Efric;    /* self-contact and friction energies */
  double Ekin;            /* kinetic energy after the corrector */
  double area, volume;    /* deformed area and enclosed volume */
  double kGauss, kMean;   /* integrated curvatures */
  uint32_t Nc;            /* contacts with penetration */
  uint32_t n_pairs;       /* contact candidates in the list */
  double Ecav;            /* cavity contact energy */
  double cavity_force;    /* sum of the cavity normal forces */
  uint32_t Nc_cav;        /* nodes penetrating the cavity */
  uint32_t pad;
} shl_energies;

/* Summary of shl_step(). */
typedef struct shl_step_report {
  uint32_t steps_done;     /* steps completed (stops early on status >= SHL_STOP_SIM) */
  int32_t worst_problem;   /* max over the steps, ShellSystem::register_problem */
  double time;             /* simulation time after the last step */
  double du_sum;           /* linked-cell displacement budget (ShellSystem.C:2634) */
  uint32_t n_rebuilds;     /* candidate-list rebuilds performed */
  uint32_t rejections;     /* repeated attempts (adaptive dt, ShellSystem.C:1104-1117) */
  shl_energies last;       /* measurements of the last step */
  /* dt-weighted sums over the steps (the MovingAverage inputs, ShellSystem.C:2830-2843) */
  double sum_dt, sum_area, sum_volume, sum_Nc, sum_Ekin, sum_Etens, sum_Ebend,
      sum_Eself, sum_Efric, sum_kGauss, sum_kMean;
  uint32_t stopped;        /* the stopping criterion became true (shl_set_stop_function) */
  uint32_t pad;
  /* dt-weighted sums of the cavity measurements (pcav = force / cavity surface) */
  double sum_pcav, sum_Nc_cav, sum_Ecav;
} shl_step_report;

typedef struct shl_ctx shl_ctx;

/* Library and build information ("shl_gb300 <version> sm_103a"). */
const char* shl_version(void);
/* Text of the last error on this thread (CUDA error string or argument check). */
const char* shl_last_error(void);
/* Human-readable name of a status. */
const char* shl_status_string(shl_status s);

/* A batch of independent shells advanced together (one context over the
 * union of the meshes; no counterpart in the reference, which runs one shell
 * per process).  Each shell has its own mesh and material/damping/thickness;
 * dt, the Newmark parameters, the precision and the pressure basis are
 * shared.  The pressure of shell k in a step is pressure_scale[k] times the
 * step's value (its ramp).  Bulk-modulus pressure is evaluated for single
 * shells only (rejected here); self-contact is per shell (below).  State vectors of a batch
 * are the shells' node-major vectors concatenated; shl_batch_layout gives the
 * node and face offsets (n_shells + 1 entries each).  Energies and the volume
 * reported by shl_step are batch totals. */
shl_status shl_batch_create(const shl_mesh* meshes, const shl_params* params, const double* pressure_scale,
                            uint32_t n_shells, shl_ctx** out);
shl_status shl_batch_layout(shl_ctx* ctx, uint32_t* n_shells, uint32_t* node_offsets, uint32_t* face_offsets);
/* Self-contact in a batch: every shell keeps its own linked cells -- its own
 * rebuild trigger (check_increment, ShellSystem.C:2591-2652), bounds, cell
 * size, d_max and cell grid (ShellSystem.C:1910-2135) -- so each shell's
 * candidate list and contact forces are those of the shell run alone; the
 * grids share one counting sort.  Shells must share the contact mode, the
 * friction coefficients, the contact damping, the cell margin and a fixed dt.
 * shl_batch_contact_stats gives each shell's du_sum and the number of its
 * candidate-list rebuilds since creation (n_shells entries; either pointer may
 * be NULL).  Pairs reported by shl_get_contact_pairs use batch face ids.
 * No counterpart in the reference, which runs one shell per process. */
shl_status shl_batch_contact_stats(shl_ctx* ctx, double* du_sum, uint32_t* n_rebuilds);

/* Set-up: ShellSystem::set_parameters + build_cache + compute_mass_damping
 * (ShellSystem.C:170-418, 490-681, 762-852).  Computes the subdivision basis,
 * the reference metrics, masses, damping and the topological neighbourhood on
 * the host and uploads everything to the current CUDA device. */
shl_status shl_create(const shl_mesh* mesh, const shl_params* params, shl_ctx** out);
void shl_destroy(shl_ctx* ctx);

/* ShellSystem::apply_initial_conditions without a load file
 * (ShellSystem.C:855-905): u = u0, v = a = 0, time = t0; computes the element
 * bounding boxes, the enclosed volume, the first contact list, and
 * a = M^-1 f at time t0 + dt with the given pressure. */
shl_status shl_apply_initial_conditions(shl_ctx* ctx, const double* u0, double t0,
                                        double pressure_next);

/* State in and out (ShellSystem::save/load, ShellSystem.C:2956-3153).
 * shl_set_state also sets u_pred = u.  When u, v and a all lie in page-locked
 * host memory mapped into the device (cudaHostAlloc), one kernel reads or
 * writes them over the host link; other pointers are copied. */
shl_status shl_set_state(shl_ctx* ctx, const double* u, const double* v, const double* a);
shl_status shl_get_state(shl_ctx* ctx, double* u, double* v, double* a);
shl_status shl_set_time(shl_ctx* ctx, double time, uint32_t time_step);
shl_status shl_get_time(shl_ctx* ctx, double* time, uint32_t* time_step);

/* Force evaluation at a given predicted state: steps 3-8 of one advance()
 * (ShellSystem.C:993-1008): candidate-list update if due, deformed metrics,
 * external force (pressure at `pressure`, self-contact with friction using
 * the current velocity), minus the internal force.  f_out gets f before the
 * damping term (may be NULL); a_out gets M^-1 (f - C v_pred) (may be NULL).
 * The stored u, v, a are not changed; the contact state is updated as the
 * reference does. */
shl_status shl_eval_forces(shl_ctx* ctx, const double* u_pred, const double* v_pred,
                           double pressure, double* f_out, double* a_out, shl_energies* e);

/* n_steps calls of ShellSystem::advance (ShellSystem.C:952-1122); with
 * adapt_dt_every > 0 each call may repeat its step with a smaller dt, and the
 * table entry of a step is used for all of its attempts.
 * pressure_table: pressure for each step (evaluated by the host at the step's
 * time t + dt), or NULL to use params.pressure.  The steps run on the
 * device without host synchronisation (captured in a CUDA graph when
 * use_graph != 0); problems are recorded per step and the remaining steps are
 * skipped once a problem >= SHL_STOP_SIM is registered.  Graph steps with a
 * fixed dt are fused (each corrector also predicts the next step; the
 * corrector's candidate-list pass, if due, is made at the start of the next
 * step); the results are bit for bit those of use_graph = 0, and every call
 * that returns or reads the state (this one, shl_step_collect, the getters of
 * the contact state, the setters) first completes a pending pass. */
shl_status shl_step(shl_ctx* ctx, uint32_t n_steps, const double* pressure_table,
                    int use_graph, shl_step_report* report);

/* Asynchronous stepping for drivers that overlap host work (and for timing
 * with CUDA events on the context's stream):
 *  shl_get_stream      the context's cudaStream_t (as void*);
 *  shl_upload_pressure_table  copy n per-step pressures to the device and
 *                      restart the table at its first entry;
 *  shl_step_enqueue    enqueue n steps (graph replays) without synchronising;
 *                      step k uses table entry k since the last upload;
 *  shl_step_collect    wait for the stream and fill the report of every step
 *                      enqueued since the last collect (or shl_step); it also
 *                      completes a candidate-list pass that the last enqueued
 *                      step left pending (see shl_step). */
shl_status shl_get_stream(shl_ctx* ctx, void** stream);
shl_status shl_upload_pressure_table(shl_ctx* ctx, const double* pressure_table, uint32_t n);
shl_status shl_step_enqueue(shl_ctx* ctx, uint32_t n_steps);
shl_status shl_step_collect(shl_ctx* ctx, shl_step_report* report);

/* Kernel timing for the roofline report: launches one kernel of the step
 * `reps` times at the current state on the context's stream, each launch
 * bracketed by CUDA events, optionally after writing `flush_bytes` of a
 * scratch buffer to evict L2; returns the mean launch time.
 * which: 0 element kernel, 1 gather/corrector (evaluation mode),
 * 2 contact force, 3 predictor. */
shl_status shl_time_kernel(shl_ctx* ctx, int which, int reps, size_t flush_bytes, double* avg_ms);
/* Per-phase timing of one step (the step is taken: the state advances):
 * the phases of advance() are launched directly, with CUDA events between
 * them, after evicting L2 with a write of flush_bytes (0 = no eviction).
 * ms_out[0..6]: predictor, linked-cell pass 1, element forces, contact forces,
 * gather + corrector, linked-cell pass 2, volume + end of step.  This is the
 * tracing counterpart of the reference's PERFLOG_START/STOP scopes
 * (macros.h:81-88). */
shl_status shl_profile_step(shl_ctx* ctx, double pressure, size_t flush_bytes, double* ms_out);

/* FP64 fused-multiply-add throughput of the current device, measured with a
 * register-resident DFMA loop (TFLOP/s, 2 flops per DFMA). */
shl_status shl_measure_fp64_peak(double* tflops);

/* Contact candidate list, sorted by (eid1, eid2), eid1 < eid2. */
shl_status shl_get_contact_pairs(shl_ctx* ctx, uint32_t* pairs /* 2*cap */, size_t cap,
                                 size_t* n_pairs);
/* Full per-pair state for checkpoints and parity checks. Any pointer may be NULL. */
shl_status shl_get_contact_state(shl_ctx* ctx, uint32_t* pairs, uint8_t* stick,
                                 double* spring_origin /* 3*cap */, double* d2, size_t cap,
                                 size_t* n_pairs, double* du_sum);
shl_status shl_set_contact_state(shl_ctx* ctx, const uint32_t* pairs, const uint8_t* stick,
                                 const double* spring_origin, const double* d2, size_t n_pairs,
                                 double du_sum);
/* SMOOTH contact: per pair (same order as shl_get_contact_state) the limit
 * surfaces' closest-point coordinates (v1, w1, v2, w2) in each face's patch
 * frame (the face's irregular vertex first), which the next step's search starts
 * from (SmoothShellShellContact::v, w, SmoothShellShellContact.C:9-14, 38-44).
 * shl_set_contact_state resets them to 1/3; shl_set_contact_coords sets them
 * (n_pairs must equal the current pair count). */
shl_status shl_get_contact_coords(shl_ctx* ctx, double* x /* 4*cap */, size_t cap, size_t* n_pairs);
shl_status shl_set_contact_coords(shl_ctx* ctx, const double* x, size_t n_pairs);
/* Force a rebuild of the candidate list at the current positions
 * (compute_shell_shell_contact_candidates(true), ShellSystem.C:1910). */
shl_status shl_rebuild_contacts(shl_ctx* ctx);

/* Per-element kGauss/kMean/etens/ebend densities of the last force
 * evaluation (ShellSystem.C:1299-1300, 2783-2784); any pointer may be NULL. */
shl_status shl_get_element_fields(shl_ctx* ctx, double* kGauss, double* kMean, double* etens,
                                  double* ebend, double* area);

/* Element-kernel variants (launch shape; for FP64, the arithmetic of the two
 * basis contractions): shl_create times the shapes of the context's path on
 * its mesh and keeps the fastest (autotuning).  shl_set_element_variant forces
 * one (0-10 FP64, 11-13 FP32; 0 and 5 keep the displacement contraction in
 * FP64, 6-10 compute in double-float, 10 in one round of faces: one block of
 * 544 threads per SM, a face per thread) or, with -1, tunes again; shl_get_element_variant
 * returns the choice, its name and the tuning times of all
 * SHL_ELEMENT_VARIANTS (ms, 0 = not timed; tuned_ms holds that many floats).
 * No counterpart in the reference. */
enum { SHL_ELEMENT_VARIANTS = 14 };
shl_status shl_set_element_variant(shl_ctx* ctx, int variant);
shl_status shl_get_element_variant(shl_ctx* ctx, int* variant, char* name, size_t cap, float* tuned_ms);

/* Scale the damping coefficients of the following steps by `factor` (relative
 * to those of the parameters; 1 restores them).  No counterpart in the
 * reference; used by relaxation schemes that smooth a starting field with
 * heavy damping before relaxing it. */
shl_status shl_scale_damping(shl_ctx* ctx, double factor);

/* Lumped inverse masses and damping coefficients (ShellSystem.C:762-852). */
shl_status shl_get_mass_damping(shl_ctx* ctx, double* Minv, double* C);

/* Relative residual of the stored state, per shell (one value for a single
 * shell, n_shells for a batch): ||f_ext - f_int||_2 / ||f_ext||_2 with
 * f_ext the pressure force at `pressure` (times each shell's pressure scale)
 * and f_int the internal force, at u (no damping, no inertia; self-contact
 * forces are not included), each vector without its rigid-translation part
 * (the resultant spread by nodal mass): the discrete pressure load of a
 * closed shell has a small resultant that moves a free shell at constant
 * speed instead of deforming it.  f2 / fext2 (may be NULL) get the squared norms.
 * flags: SHL_RESIDUAL_FP64 evaluates the forces in FP64 also in an FP32
 * context; SHL_RESIDUAL_CORRECT (FP32 context, with FP64) also stores the
 * defect f64 - f32 at this state, which the following steps add to their FP32
 * force (mixed-precision defect correction, so relaxation converges to the
 * FP64 equilibrium); SHL_RESIDUAL_CLEAR drops a stored defect;
 * SHL_RESIDUAL_CONTACT (self-contact on, no friction) adds the self-contact
 * force of the current candidate list to f_int (its static part: the penalty
 * force of ShellSystem.C:1803-1900 without the contact damping), for
 * equilibria held by contact; the contact state is not changed.
 * No counterpart in the reference, which has no residual stop. */
enum { SHL_RESIDUAL_FP64 = 1, SHL_RESIDUAL_CORRECT = 2, SHL_RESIDUAL_CLEAR = 4, SHL_RESIDUAL_CONTACT = 8 };
shl_status shl_residual(shl_ctx* ctx, double pressure, int flags, double* rel, double* f2, double* fext2);

/* The pressure as a config expression of t (the muparser language of the
 * config file: operators, functions, pi; d reads 0): compiled on the host and
 * evaluated by the device at each step's time t + dt, in place of the
 * per-step table (ShellSystem.C:934-936).  NULL or "" returns to the table.
 * shl_eval_pressure_function evaluates the compiled program at n times (a
 * check of the device evaluation). */
shl_status shl_set_pressure_function(shl_ctx* ctx, const char* expr);
shl_status shl_eval_pressure_function(shl_ctx* ctx, const double* t, uint32_t n, double* out);

/* Cavity semi-axes as config expressions of t (Rx, Ry, Rz of config.cfg),
 * evaluated by the device at each step's time (ShellSystem.C:194-196,
 * 421-470); NULL or "" keeps the constant of the parameters. */
shl_status shl_set_cavity_functions(shl_ctx* ctx, const char* rx, const char* ry, const char* rz);

/* Static-friction spring origins of the cavity contacts, 3 per node (the
 * NodeCache::spring_origin of save/load, ShellSystem.C:2976-2980, 3073-3076);
 * zeros without cavity contact. */
shl_status shl_get_cavity_origins(shl_ctx* ctx, double* origins);
shl_status shl_set_cavity_origins(shl_ctx* ctx, const double* origins);

/* The current time step (adaptive dt: the next attempt's) and the repeated
 * attempts since the last report. */
shl_status shl_get_dt(shl_ctx* ctx, double* dt, uint32_t* rejections);
/* Stopping criterion as a config expression of t (shell.C:314-318), tested on
 * the device after every step; shl_step returns early with report->stopped
 * set once it is nonzero.  NULL or "" removes it. */
shl_status shl_set_stop_function(shl_ctx* ctx, const char* expr);

/* Measurements of the last force evaluation or step (the scalars of
 * measure_properties, ShellSystem.C:2714-2846). */
shl_status shl_get_energies(shl_ctx* ctx, shl_energies* e);

/* Node and face counts, and the mesh the context was made from (file order,
 * reference positions). */
shl_status shl_context_size(shl_ctx* ctx, uint32_t* n_nodes, uint32_t* n_faces);
shl_status shl_context_mesh(shl_ctx* ctx, double* xyz /* 3V */, uint32_t* faces /* 3F */);

/* Per-node measurement vectors of the last step (node_vectors of
 * ShellSystem.C:126-130): kinetic energy density (Ekin_node / mean area of the
 * incident faces, 2796-2812), cavity-contact energy density (1630), self-contact
 * and friction energy densities (1699, 1862-1877) and nodal mass.  V values each; any pointer may be NULL. */
shl_status shl_get_node_fields(shl_ctx* ctx, double* ekin, double* ecav, double* eself, double* efric,
                               double* mass);

/* ShellSystem::apply_initial_conditions with a load file (ShellSystem.C:855-888)
 * after shl_set_state / shl_set_time / shl_set_contact_state: positions,
 * bounding boxes, a forced candidate-list build that keeps the loaded pairs,
 * deformed metrics, and volume0 = the loaded state's volume.  v and a are kept. */
shl_status shl_apply_loaded_state(shl_ctx* ctx);

/* ---- files (host code over the calls above) ---------------------------- */

/* State file of shell.C:383-390 + ShellSystem::save (ShellSystem.C:2956-3032),
 * 17 significant digits: time_step, dt, time, wall_time; per node
 * "ux vx ax uy vy ay uz vz az sx sy sz" (s = cavity spring origin, 0 here);
 * the number of measurement rows and the rows (14 columns each, avg_rows
 * row-major: dt, area, vol, pcav, Nc_cav, Nc, Ekin, Etens, Ebend, Ecav, Eself,
 * Efric, kGauss, kMean, each weighted with dt); the sticking self-contacts
 * "eid1 eid2 ox oy oz". */
shl_status shl_save_state_file(shl_ctx* ctx, const char* path, uint32_t time_step, double dt,
                               double wall_time, const double* avg_rows, uint32_t n_rows);
/* Reads such a file into the context (u, v, a, time, time_step, sticking
 * contacts) and calls shl_apply_loaded_state.  Returns the file's time step,
 * dt and wall time, and up to cap_rows measurement rows (SHL_ERR_CAPACITY if
 * the file holds more); avg_rows may be NULL. */
shl_status shl_load_state_file(shl_ctx* ctx, const char* path, uint32_t* time_step, double* dt,
                               double* wall_time, double* avg_rows, uint32_t cap_rows, uint32_t* n_rows);
/* ASCII VTK unstructured grid of ShellSystem::write_vtk (ShellSystem.C:3156-3320):
 * reference positions, point data ux uy uz ecav efric ekin eself mass, cell
 * data ebend etens kGauss kMean of the last step. */
shl_status shl_write_vtu(shl_ctx* ctx, const char* path);

/* ---- host helpers of the driver (no device work) ----------------------- */

/* Closed icosphere: the 20-face icosahedron refined `level` times, each
 * midpoint pushed to the unit sphere, written as OFF text with %g and read
 * back (so ids and rounded coordinates equal those of icosasphere<level>.off).
 * Writes up to cap_nodes nodes and cap_faces faces; returns the counts. */
shl_status shl_icosphere(uint32_t level, double* xyz, size_t cap_nodes, uint32_t* faces,
                         size_t cap_faces, uint32_t* n_nodes, uint32_t* n_faces);
/* The OFF text of shl_icosphere(level) into buf (NUL terminated); *len gets
 * the length needed (call with buf = NULL to query). */
shl_status shl_icosphere_off(uint32_t level, char* buf, size_t cap, size_t* len);
/* Read an OFF file (triangles only). */
shl_status shl_read_off(const char* path, double* xyz, size_t cap_nodes, uint32_t* faces,
                        size_t cap_faces, uint32_t* n_nodes, uint32_t* n_faces);

/* Seeded imperfection u_i = amplitude * g_i * x_i/|x_i|, g_i ~ N(0,1) from
 * Philox-4x32-10 (key = seed, counter = node id) with a Box-Muller map. */
shl_status shl_gaussian_normal_imperfection(const double* xyz, uint32_t n_nodes, double amplitude,
                                            uint64_t seed, double* u_out);

/* Force evaluation that allocates no device memory, for callers that cannot
 * call cudaMalloc when they evaluate forces: code that runs inside its own
 * CUDA stream capture (allocation is not allowed there), and hosts whose
 * device memory all comes from an arena they own and that forbid allocation
 * on their time-stepping path.  No counterpart in the reference.
 *
 * f_dev (3*n_nodes doubles, device) receives f = pressure force - internal
 * force at the predicted displacement u_dev (3*n_nodes doubles, device), as
 * f_out of shl_eval_forces for a shell without self-contact and with
 * bulk_modulus = 0 (both are rejected here).  Only the context's constant
 * set-up data are read; its state, buffers and step prediction are untouched.
 * The per-(face, patch node) force shares go to a scratch array compiled into
 * the library: a static device array of 12 * 32768 slots of 3 doubles (9 MiB)
 * that every GPU which loads the library holds until the process exits.  A
 * face of a 12-node patch takes 12 slots, so shells of up to 32768 faces of
 * regular patches fit; patches around vertices of valence N take N + 6 slots.
 * Shells with more slots are rejected with SHL_ERR_CAPACITY.  The call must
 * be made with the context's device current (else SHL_ERR_ARG).
 *
 * The first call on a device looks up the scratch address there (and may
 * make the CUDA runtime load the library's device code); make that first call
 * before any stream capture.  All calls share the one scratch array, so calls
 * that overlap on the GPU (different streams, or different contexts on one
 * device) race and must be ordered by the caller.  stream: a cudaStream_t, or
 * NULL for the default stream; the call does not synchronise. */
shl_status shl_internal_force_noalloc(shl_ctx* ctx, const double* u_dev, double pressure, double* f_dev,
                                      void* stream);

/* ---- warm-start surrogate (no counterpart in the reference) ------------ */

/* A multilayer perceptron dims[0] -> dims[1] -> ... -> dims[n_dims-1], GELU
 * after every layer but the last, trained and evaluated on the GPU by the
 * library's own BF16 tensor-core kernels (FP32 accumulation, FP32 master
 * weights, Adam).  Weights are row-major (out x in) FP32 on the host side. */
typedef struct shl_mlp shl_mlp;
shl_status shl_mlp_create(const uint32_t* dims, uint32_t n_dims, uint32_t max_batch, uint64_t seed,
                          shl_mlp** out);
void shl_mlp_destroy(shl_mlp* mlp);
shl_status shl_mlp_set_params(shl_mlp* mlp, uint32_t layer, const float* W, const float* b);
shl_status shl_mlp_get_params(shl_mlp* mlp, uint32_t layer, float* W, float* b);
/* Training set: n rows of inputs (dims[0]) and targets (dims[last]), copied to the device. */
shl_status shl_mlp_set_dataset(shl_mlp* mlp, const float* X, const float* T, uint64_t n);
/* iters Adam steps on shuffled mini-batches (mean squared error), learning
 * rate decayed from lr0 to lr_final on a cosine; the loss of every
 * curve_every-th batch goes to loss_curve (ceil(iters / curve_every) values). */
shl_status shl_mlp_train(shl_mlp* mlp, uint32_t iters, uint32_t batch, float lr0, float lr_final, uint64_t seed,
                         float* loss_curve, uint32_t curve_every);
/* Outputs for n input rows (host arrays). */
shl_status shl_mlp_predict(shl_mlp* mlp, const float* X, uint32_t n, float* Y);
/* Loss and gradients of one batch of n <= max_batch rows (no update);
 * dW[l] (out x in) and db[l] may be NULL. */
shl_status shl_mlp_gradients(shl_mlp* mlp, const float* X, const float* T, uint32_t n, double* loss,
                             float* const* dW, float* const* db);
/* C = A . B^T with the library's BF16 GEMM: A (M x K) and B (N x K) as BF16
 * bit patterns, K a multiple of 8; C is M x N FP32. */
shl_status shl_gemm_bf16(const uint16_t* A, const uint16_t* B, uint32_t M, uint32_t N, uint32_t K, float* C);
/* Average device time (ms, CUDA events over `reps` launches after a warm-up) of
 * the same GEMM on device-resident operands of the given shape (pseudo-random
 * values), for throughput figures. */
shl_status shl_gemm_bf16_time(uint32_t M, uint32_t N, uint32_t K, int reps, double* avg_ms);

/* Default parameters (ShellSystem constructor and set_parameters defaults). */
void shl_params_default(shl_params* p);

#ifdef __cplusplus
}
#endif

#endif /* SHL_H_ */
