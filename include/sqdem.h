/* sqdem.h — C ABI of libsqdem_gpu.so, the GB300 (sm_103a) engine for SudoDEM3D's
 * superellipsoid per-timestep path.
 *
 * One context = one GPU scene (bodies, materials, contact table, collider state) living
 * in device memory.  A call to sqdem_step() advances it by whole timesteps with the same
 * engine sequence a SudoDEM3D script builds with
 *
 *   O.engines = [ForceResetter(),
 *                InsertionSortCollider([Bo1_Superquadrics_Aabb(), Bo1_Wall_Aabb()], verletDist=...),
 *                InteractionLoop([Ig2_Wall_Superquadrics_SuperquadricsGeom(),
 *                                 Ig2_Superquadrics_Superquadrics_SuperquadricsGeom()],
 *                                [Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys()],
 *                                [SuperquadricsLaw()]),
 *                NewtonIntegrator(damping=..., gravity=..., isSuperquadrics=1)]
 *
 * Conventions: plain pointers and sizes, no exceptions across the ABI, every call returns
 * an sqdem_status; host buffers are owned by the caller, device buffers by the library.
 * Body ids are the reference's Body::id (walls and particles share one id space).
 *
 * Reference interfaces replaced (paths relative to the SudoDEM repository root):
 *   Scene::moveToNextTimeStep                 SudoDEM3D/core/Scene.cpp:70-138
 *   Engine::action (the four engines above)   SudoDEM3D/core/Engine.hpp:33-34
 *   BoundFunctor::go / IGeomFunctor::go /
 *   IPhysFunctor::go / LawFunctor::go         SudoDEM3D/pkg/common/Dispatching.hpp:19-71
 *   O.bodies / O.interactions / O.forces      SudoDEM3D/py/wrapper/sudodemWrapper.cpp:937-987
 */
#ifndef SQDEM_H
#define SQDEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sqdem_ctx sqdem_ctx;
typedef struct sqdem_batch sqdem_batch;

typedef enum {
  SQDEM_OK = 0,
  SQDEM_ERR_ARG = 1,      /* bad argument (size, pointer, range) */
  SQDEM_ERR_CUDA = 2,     /* a CUDA runtime call failed; see sqdem_last_error */
  SQDEM_ERR_CAPACITY = 3, /* contact table / candidate buffer overflow; state not advanced past it */
  SQDEM_ERR_STATE = 4,    /* call out of order (e.g. step before bodies are set) */
  SQDEM_ERR_NUMERIC = 5   /* NaN depth met (the reference calls exit(1), Superquadrics.cpp:1352) */
} sqdem_status;

/* Body kinds. */
enum { SQDEM_SUPERQUADRIC = 0, SQDEM_WALL = 1 };

/* Arithmetic form of the narrowphase. */
enum { SQDEM_FP64 = 0, SQDEM_MIXED = 1 };

/* Contact model (the functor set of the InteractionLoop):
 *   SQDEM_CONTACT_LINEAR         Ig2_Wall_Superquadrics_SuperquadricsGeom, Ig2_Superquadrics_
 *                                Superquadrics_SuperquadricsGeom (Levenberg-Marquardt),
 *                                Ip2_SuperquadricsMat_SuperquadricsMat_SuperquadricsPhys,
 *                                SuperquadricsLaw                      (the default)
 *   SQDEM_CONTACT_HERTZ_MINDLIN  Ig2_Wall_Superquadrics_SuperquadricsGeom2, Ig2_Superquadrics_
 *                                Superquadrics_SuperquadricsGeom2 (Nelder-Mead),
 *                                Ip2_SuperquadricsMat2_SuperquadricsMat2_HertzMindlinPhys,
 *                                SuperquadricsLaw2
 *                                (pkg/dem/Superquadrics_Ig2.cpp:1624-1878, 2322-2517, 2615-2700;
 *                                 pkg/dem/Superquadrics.cpp:974-1013, 1118-1160, 1367-1557)
 * The Hertz-Mindlin search always runs in FP64 (sqdem_config.precision applies to the linear
 * model's search). */
enum { SQDEM_CONTACT_LINEAR = 0, SQDEM_CONTACT_HERTZ_MINDLIN = 1 };

typedef struct {
  int device;              /* CUDA device ordinal */
  int precision;           /* SQDEM_FP64 or SQDEM_MIXED */
  int contacts_per_body;   /* contact-table capacity per particle (0 -> 16) */
  int use_graph;           /* capture the timestep in a CUDA graph (1) or launch eagerly (0) */
} sqdem_config;

/* Engine attributes, named as in the reference:
 *   NewtonIntegrator.{damping,gravity,isSuperquadrics,exactAsphericalRot}  NewtonIntegrator.hpp:70-89
 *   InsertionSortCollider.{verletDist,targetInterv,minSweepDistFactor,sortAxis}
 *                                                       InsertionSortCollider.hpp:212-222
 *   Scene.dt                                            core/Scene.hpp */
typedef struct {
  double dt;
  double gravity[3];
  double damping;
  double verletDist;
  int targetInterv;
  double minSweepDistFactor;
  int sortAxis;
  int isSuperquadrics;
  int exactAsphericalRot;
} sqdem_params;

/* Per-step error words read back by sqdem_sync (the reference logs NaN normals/forces to
 * SuperquadricsLaw_err.log, Superquadrics_Ig2.cpp:2165-2188, Superquadrics.cpp:1324-1350). */
typedef struct {
  long long nan_normals;      /* NaN contact normals met by the narrowphase */
  long long nan_forces;       /* NaN forces zeroed by the contact law */
  long long lm_calls;         /* Levenberg-Marquardt solves */
  long long lm_iterations;    /* summed LM iterations */
  long long lm_maxiter;       /* solves that hit itmax (stop code 3) */
  long long overflow;         /* contact-table or candidate-buffer overflows */
  long long collider_runs;    /* collider passes executed */
  long long steps;            /* timesteps executed */
  long long evals_fp32;       /* Disfunction evaluations on the FP32 pipes (double-float, mixed form) */
  long long evals_fp64;       /* Disfunction evaluations in FP64 */
  long long lm_rounds_max;    /* longest contact, in evaluation rounds of the LM kernel
                                 (the critical path of the contact stage), max over steps */
  long long fallback_fp64;    /* mixed form: searches deferred to the FP64 kernel (a decision
                                 inside its rounding band, itmax reached, or an evaluation it does
                                 not reproduce) */
  long long lm_rounds_max_ff; /* mixed form: longest search in rounds of the double-float kernel
                                 (lm_rounds_max: of the FP64 kernel) */
  long long long_queue;       /* searches of 32+ iterations at the previous step, queued for the
                                 FP64 kernel's long-search handling (both forms) */
} sqdem_report;

/* Record layouts shared with the CPU oracle (doubles per record). */
#define SQDEM_BODY_STRIDE 37
/* pos3 ori4(w,x,y,z) vel3 angVel3 angMom3 force3 torque3 bmin3 bmax3 refPos3
   sweepLength lastUpdateIter mass inertia3 */
#define SQDEM_INTR_STRIDE 57
/* id1 id2 isReal hasGeom depth contactAngle2 contactPoint3 normal3 shearInc3 point1_3 point2_3
   isShearNew kn ks tanphi normalForce3 shearForce3 twist3 orthonormal3 relVn3 relVs3 cellDist3
   curvatures1_2 curvatures2_2 curvatureAngle alpha K E curvatures_sum isSphere
   (the last ten: SuperquadricsGeom2, Hertz-Mindlin model; zero under the linear model) */
#define SQDEM_SCALARS 9
/* iter maxVelocitySq fastestBodyMaxDist strideActive newtonFound verletDist numReinit colliderRuns
   sortedBoundsValid (0: the next collider pass is a full sort, InsertionSortCollider.cpp:213-222) */

/* Create a context on cfg->device.  Replaces building a Scene (core/Scene.hpp). */
sqdem_status sqdem_create(sqdem_ctx** out, const sqdem_config* cfg);
void sqdem_destroy(sqdem_ctx* ctx);
/* Last error text of this context (static storage valid until the next call). */
const char* sqdem_last_error(sqdem_ctx* ctx);

/* Materials, SuperquadricsMat{Kn,Ks,frictionAngle,betan,betas,density}
 * (pkg/dem/Superquadrics.hpp:247-264).  Index i is the material id used below. */
sqdem_status sqdem_set_materials(sqdem_ctx* ctx, int n, const double* Kn, const double* Ks,
                                 const double* frictionAngle, const double* betan,
                                 const double* betas, const double* density);

/* All bodies in reference id order.  kind[i] is SQDEM_SUPERQUADRIC or SQDEM_WALL.
 * shape5 = (rx,ry,rz,eps1,eps2) for superquadrics (ignored for walls); wall = (axis,sense)
 * (ignored for particles); state = SQDEM_BODY_STRIDE doubles per body (force/torque and bound
 * columns are ignored: bounds start unset, as after NewSuperquadrics_rot2 and utils.wall,
 * py/_superquadrics_utils.cpp:354-380, py/utils.py:311-327).  Mass and inertia are taken
 * from the state columns; sqdem_shape_props gives the reference's values.  At most 64 walls
 * (SQDEM_ERR_CAPACITY beyond). */
sqdem_status sqdem_set_bodies(sqdem_ctx* ctx, int n, const int* kind, const double* shape5,
                              const int* wall_axis_sense, const int* mat, const int* isSphere,
                              const double* state);
sqdem_status sqdem_set_params(sqdem_ctx* ctx, const sqdem_params* p);

/* Launch shapes of the contact stage: resident blocks per SM of the search kernel (at most
 * what its occupancy allows) and grid-stride blocks per SM of the first contact pass; 0 keeps
 * the default.  Shapes change no result, only the time. */
sqdem_status sqdem_set_launch_shape(sqdem_ctx* ctx, int search_blocks_per_sm, int pass1_blocks_per_sm);
typedef struct {
  int search_blocks_per_sm, pass1_blocks_per_sm;   /* the shape chosen and set */
  double ms_per_step;                               /* its device time per step */
  int candidates;                                   /* shapes timed */
} sqdem_tune;
/* Autotuner: times each candidate shape (search blocks per SM 1..occupancy x pass-1 blocks
 * per SM 4/8/16/32) for `steps` timesteps on the scene itself, twice, and sets the fastest.
 * The tuning steps are ordinary timesteps (shapes change no result): the scene advances by
 * candidates x (2 x steps + 1) steps.  No counterpart in the reference. */
sqdem_status sqdem_autotune(sqdem_ctx* ctx, int steps, sqdem_tune* out);

/* Contact model (SQDEM_CONTACT_*); takes effect at the next step, existing contacts keep
 * their state.  sqdem_contact_model returns the current one (-1 for a NULL context). */
sqdem_status sqdem_set_contact_model(sqdem_ctx* ctx, int model);
int sqdem_contact_model(sqdem_ctx* ctx);
/* Number of materials set (0 before sqdem_set_materials). */
int sqdem_num_materials(sqdem_ctx* ctx);
/* SuperquadricsMat2{G, nu} (pkg/dem/Superquadrics.hpp:266-277) per material, n = the count
 * given to sqdem_set_materials; defaults G = 29e9 Pa, nu = 0.15.  Used by the Hertz-Mindlin
 * model only. */
sqdem_status sqdem_set_material_moduli(sqdem_ctx* ctx, int n, const double* G, const double* nu);
sqdem_status sqdem_get_material_moduli(sqdem_ctx* ctx, double* G, double* nu);

/* Advance nsteps timesteps (asynchronous on the context stream). */
sqdem_status sqdem_step(sqdem_ctx* ctx, int nsteps);
/* Wait for the stream, read and clear the error words.  report may be NULL. */
sqdem_status sqdem_sync(sqdem_ctx* ctx, sqdem_report* report);

/* Body state in the SQDEM_BODY_STRIDE layout (O.bodies[i].state, O.forces). */
sqdem_status sqdem_get_body_state(sqdem_ctx* ctx, double* out);
/* Overwrite dynamic and bound state from the same layout (mass/inertia/force columns ignored). */
sqdem_status sqdem_put_body_state(sqdem_ctx* ctx, const double* in);
/* Same as get/put but only positions, orientations, velocities, angular velocities and
 * angular momenta (16 doubles per body), for streaming state to and from the host. */
sqdem_status sqdem_get_kinematics(sqdem_ctx* ctx, double* out16);
sqdem_status sqdem_put_kinematics(sqdem_ctx* ctx, const double* in16);

/* Interactions (O.interactions): count, then records in the SQDEM_INTR_STRIDE layout.
 * include_potential = 0 returns only real interactions (geom and phys present). */
sqdem_status sqdem_num_interactions(sqdem_ctx* ctx, int include_potential, long* n);
sqdem_status sqdem_get_interactions(sqdem_ctx* ctx, int include_potential, double* out, long cap, long* n);
/* Replace the contact table (history included) from records. */
sqdem_status sqdem_put_interactions(sqdem_ctx* ctx, long n, const double* in);

sqdem_status sqdem_get_scalars(sqdem_ctx* ctx, double* out9);
sqdem_status sqdem_put_scalars(sqdem_ctx* ctx, const double* in9);

/* Record the full contact geometry (point1/2, shearInc, twist/orthonormal axes, relative
 * velocities of SuperquadricsGeom, Superquadrics.hpp:175-208) every step.  Off by default:
 * the step then writes only the history the next step needs. */
sqdem_status sqdem_set_record_full(sqdem_ctx* ctx, int on);

/* Schedule of the Levenberg-Marquardt evaluations (no counterpart in the reference, which
 * runs one search per thread).  on = 1 (default): once the contact queue is drained, lanes
 * without a contact evaluate the points the searches still running in their warp will ask
 * for next; on = 0: every lane evaluates only its own search's point.  Results are identical
 * bit for bit; only the time of the longest searches changes. */
sqdem_status sqdem_set_lm_spread(sqdem_ctx* ctx, int on);

/* Periodic-boundary correction, off by default (the reference's behaviour).  For a contact
 * with the image of body 2 (cellDist != 0) the reference applies body 2's torque about its
 * unshifted position (pkg/dem/Superquadrics.cpp:1356, its own FIXME at :1550) and leaves the
 * image's field velocity velGrad*shift2 out of the relative velocity (:1042-1045); under
 * compression these spin boundary particles up without bound.  on = 1 takes the torque arm
 * from the image and adds velGrad*shift2 (both models' geometry, the linear law's torque).
 * No counterpart in the reference. */
sqdem_status sqdem_set_periodic_fix(sqdem_ctx* ctx, int on);

/* Device time (ms, summed over the steps of the last sqdem_step call made with use_graph = 0,
 * CUDA events on the context stream) of the contact search kernel (k_contacts_lm, or the mixed
 * form's double-float k_contacts_lm_ff) and of the mixed form's FP64 fallback kernel (0 for the
 * FP64 form).  Linear contact model only (0, 0 otherwise).  No counterpart in the reference
 * (per-kernel timing of what the reference times per engine with timing.stats). */
sqdem_status sqdem_search_times(sqdem_ctx* ctx, double* out2);

/* Per-stage device time of the last sqdem_step call in milliseconds (cudaEvent pairs on the
 * context stream; only when the context was created with use_graph == 0):
 * out[0] collider gate+passes, out[1] contacts (narrowphase+law), out[2] integrator+reductions. */
sqdem_status sqdem_stage_times(sqdem_ctx* ctx, double* out3);

/* Periodic cell (Scene.isPeriodic with core/Cell.hpp): hSize9 row-major, its columns are the cell
 * base vectors (Cell::setHSize); velGrad9 (may be NULL) is applied at the next integrator pass
 * (Cell::setVelGrad), homoDeform on.  Positions stay unwrapped; interactions carry cellDist and
 * shift2 = hSize*cellDist (InteractionLoop.cpp:100-106).  Walls are not supported in a periodic scene.
 * sqdem_get_cell / sqdem_put_cell: hSize9 velGrad9 prevVelGrad9 size3 prevCellSize3 (33 doubles). */
sqdem_status sqdem_set_periodic(sqdem_ctx* ctx, const double* hSize9, const double* velGrad9);
sqdem_status sqdem_set_velgrad(sqdem_ctx* ctx, const double* velGrad9);
sqdem_status sqdem_get_cell(sqdem_ctx* ctx, double* out33);
sqdem_status sqdem_put_cell(sqdem_ctx* ctx, const double* in33);

/* Replay the timestep as a CUDA graph (on = 1, default) or launch its kernels one by one with
 * per-stage event timing readable through sqdem_stage_times (on = 0). */
sqdem_status sqdem_set_use_graph(sqdem_ctx* ctx, int on);

/* Timing entry points (cudaEvents on the context stream).
 * sqdem_time_steps: nsteps timesteps, device milliseconds in *ms.
 * sqdem_time_e2e:   nsteps x (upload 16 doubles/body from host, one timestep, download to host),
 *                   the end-to-end path of a host caller; in16 and out16 alternate as source and
 *                   destination (the state of step i is the input of step i+1); use pinned buffers.
 * sqdem_time_contacts: one launch of the narrowphase+law kernel, averaged over nrep launches. */
sqdem_status sqdem_time_steps(sqdem_ctx* ctx, int nsteps, double* ms);
sqdem_status sqdem_time_e2e(sqdem_ctx* ctx, int nsteps, const double* in16, double* out16, double* ms);
sqdem_status sqdem_time_contacts(sqdem_ctx* ctx, int nrep, double* ms);

/* One pass of the contact stage (narrowphase, contact physics and law; the work of
 * sqdem_time_contacts without its timing) that allocates nothing: its work queue is a fixed
 * static device array of SQDEM_STATIC_QUEUE_MAX ints (4 MiB per GPU, held until exit) instead
 * of a buffer owned by the context.  For callers that cannot call cudaMalloc at that point
 * (host frameworks that own device memory through their own pool and forbid raw allocations
 * after start-up, loops that must not block in the allocator).  Rejects, with
 * SQDEM_ERR_CAPACITY, a context whose contact-table capacity (contacts_per_body x particles)
 * exceeds the array; the check reads only that host-side capacity.  The first call on a device
 * looks up the array's address (cudaGetSymbolAddress) and keeps it; make it before any stream
 * capture.  Calls share the array, so calls that overlap on the GPU race.  Asynchronous on the
 * context stream, ordered after the work already queued there.  No counterpart in the
 * reference. */
#define SQDEM_STATIC_QUEUE_MAX (1 << 20)
sqdem_status sqdem_contacts_static_queue(sqdem_ctx* ctx);

/* Pipe peaks of the GPU `device`, measured by kernels of known instruction mix (no counterpart
 * in the reference; the denominators of the contact stage's roofline): out[0] FP64 FMA TFLOP/s,
 * out[1] FP32 FMA TFLOP/s, out[2] FP64 Disfunction evaluations per second (1e9/s) and out[3]
 * double-float Disfunction evaluations per second (1e9/s), every lane of a full grid evaluating
 * independent points.  Allocates 64 bytes of device memory for the duration of the call. */
sqdem_status sqdem_pipe_peaks(int device, double* out4);

/* Superquadrics::Initial (pkg/dem/Superquadrics.cpp:47-93): volume, geometric inertia (3),
 * bounding radius r_max, for unit density.  Host-only helper. */
sqdem_status sqdem_shape_props(double rx, double ry, double rz, double eps1, double eps2, double* out5);

/* Number of kernel launches issued by the last sqdem_step call. */
long long sqdem_launch_count(sqdem_ctx* ctx);

/* ---------------------------------------------------------------------------------------
 * Boundary controller: CompressionEngine for a cubic specimen (pkg/dem/Compression.hpp:39-252,
 * action_cubic Compression.cpp:395-604, as compiled with SOLE_GAIN and NEW_SCHEME), run each
 * step between InteractionLoop and NewtonIntegrator.  Bodies 0-5 must be the walls left,
 * right, front, back, bottom, top.  Configuration, SQDEM_SERVO_CONFIG doubles: enabled,
 * z_servo, continueFlag, hydroStrain, shearMode, left/right/front/back/bottom/top
 * _wall_activated, iterate_num_max, solve_num_max, echo_interval, savedata_interval,
 * ramp_interval, ramp_chunks, goalx, goaly, goalz, gain_alpha, target_strain, f_threshold,
 * fmin_threshold, unbf_tol, max_vel, hydroStrainRate, width0, height0, depth0.  enabled = 0
 * removes the engine.  Setting it starts the engine afresh (its first run initialises). */
#define SQDEM_SERVO_CONFIG 30
/* Engine state, SQDEM_SERVO_STATE doubles: width, depth, height, x_area, y_area, z_area,
 * wsxx, wsyy, wszz, wsxx_left, wsxx_right, wsyy_front, wsyy_back, wszz_bottom, wszz_top,
 * gain_x, gain_x1, gain_y, gain_y1, gain_z, gain_z1, UnbalancedForce, particlesVolume,
 * Init_boxVolume, Current_boxVolume, strain[2], iterate_num, solve_num, rampNum,
 * Flag_ForceTarget, firstRun, width0, height0, depth0, stopAtIter (-1: none), quiet flag.
 * When an engine sets Scene::stopAtIter (consolidation complete, target strain reached),
 * the steps from that iteration on do nothing, as O.run stops there; sqdem_put_servo with
 * stopAtIter = -1 resumes. */
#define SQDEM_SERVO_STATE 36
sqdem_status sqdem_set_servo(sqdem_ctx* ctx, const double* config);
sqdem_status sqdem_get_servo(sqdem_ctx* ctx, double* state);
sqdem_status sqdem_put_servo(sqdem_ctx* ctx, const double* state);
/* NewtonIntegrator::quiet_system_flag (NewtonIntegrator.hpp:73): the next step zeroes all
 * velocities instead of moving the bodies, then clears the flag (NewtonIntegrator.cpp:246-299). */
sqdem_status sqdem_set_quiet(sqdem_ctx* ctx, int on);
/* Shop::unbalancedForce(useMaxForce) (pkg/dem/Shop_01.cpp:148-188) on the forces of the last
 * step; Shop::getStress(volume) (pkg/dem/Shop_02.cpp:350-376), 9 doubles row-major, volume 0
 * meaning the periodic cell's volume (1 without a cell).  Sums follow table order. */
sqdem_status sqdem_unbalanced_force(sqdem_ctx* ctx, int use_max, double* out);
sqdem_status sqdem_get_stress(sqdem_ctx* ctx, double volume, double* out9);

/* Snapshot of the whole context state as one byte blob: materials, parameters, bodies (with
 * bounds and previous-pass bounds), the contact table with its history, iteration, collider
 * and integrator bookkeeping, periodic cell and CompressionEngine.  buf = NULL returns the size
 * in *size.  sqdem_restore loads a blob into a context (any precision / capacity config; the
 * table must fit): it then continues bit for bit as the original.  Replaces O.save / O.load
 * (core/Omega.cpp:230-279) within this library; the blob is not the reference's .xml.bz2 and
 * is refused by a build whose state records differ in size. */
sqdem_status sqdem_snapshot(sqdem_ctx* ctx, void* buf, size_t* size);
sqdem_status sqdem_restore(sqdem_ctx* ctx, const void* buf, size_t size);

/* ---------------------------------------------------------------------------------------
 * Batches of independent specimens (no counterpart in the reference, which runs one Scene per
 * process): n scenes, each a full context set up through the functions above
 * (sqdem_batch_scene gives its handle), stepped together by one CUDA graph launch per step in
 * which every scene's step is a parallel branch.  A scene's results are exactly those of its
 * context stepped alone.  Changing a scene (bodies, engine) rebuilds the graph at the next
 * step.  Scenes of a batch share one device; sqdem_destroy must not be called on them. */
sqdem_status sqdem_batch_create(sqdem_batch** out, int n_scenes, const sqdem_config* cfg);
void sqdem_batch_destroy(sqdem_batch* batch);
const char* sqdem_batch_last_error(sqdem_batch* batch);
int sqdem_batch_size(sqdem_batch* batch);
sqdem_status sqdem_batch_scene(sqdem_batch* batch, int i, sqdem_ctx** ctx);
/* Advance every scene nsteps timesteps (asynchronous on the batch stream). */
sqdem_status sqdem_batch_step(sqdem_batch* batch, int nsteps);
/* Wait, read and clear every scene's error words: counters summed, lm_rounds_max the largest;
 * returns the first scene's error (e.g. SQDEM_ERR_CAPACITY). */
sqdem_status sqdem_batch_sync(sqdem_batch* batch, sqdem_report* total);
/* Device time of nsteps batch steps (graph launches, inputs resident), milliseconds. */
sqdem_status sqdem_batch_time_steps(sqdem_batch* batch, int nsteps, double* ms);
/* End to end: per step, all scenes' kinematics (16 doubles per body, scenes in order, the
 * sqdem_get_kinematics layout) copied from host in16 (alternating with out16) to the device,
 * one batch step, and copied back. */
sqdem_status sqdem_batch_time_e2e(sqdem_batch* batch, int nsteps, const double* in16, double* out16, double* ms);
/* Kernel launches of one batch step (all scenes). */
long long sqdem_batch_launch_count(sqdem_batch* batch);

/* ---------------------------------------------------------------------------------------
 * Adjoint of a window of timesteps (no counterpart in the reference, which has no
 * differentiation; the forward it differentiates is the linear contact model's step,
 * Scene::moveToNextTimeStep core/Scene.cpp:70-138 with the engines of sqdem_step).
 *
 * A window starts from a scene state (bodies and interactions in the SQDEM_BODY_STRIDE /
 * SQDEM_INTR_STRIDE layouts, e.g. from sqdem_get_body_state / sqdem_get_interactions) and
 * keeps its potential-pair set: the collider does not run and the law's bound-separation
 * erase (pkg/dem/Superquadrics.cpp:1203-1207) is not applied; contacts still open and close
 * through the narrowphase and the depth gate.  Ip2 (Superquadrics.cpp:1086-1116) is applied
 * afresh to every pair from the materials given.  Particles must be free, damped, aspherical
 * superquadrics not flagged as spheres; walls move with their prescribed velocity; no
 * periodic cell, no viscous contact damping.
 *
 * Parameters: per-body exponents eps1, eps2 (narrowphase shape; mass, inertia and r_max keep
 * the values of the state), per-material Kn, Ks and friction coefficient mu = tan(angle).
 * Loss = sum_b wF_b . F_b(last step) + wX_b . pos_b(end), F_b the body's contact force of
 * the window's last step (for a wall, its normal-force component is the wall force).
 * Gradients are those of the discrete map with every branch (Levenberg-Marquardt decisions,
 * contact gates, Coulomb cap, damping signs) taken as in the forward run. */
typedef struct sqdem_adj sqdem_adj;
sqdem_status sqdem_adj_create(sqdem_adj** out, int device);
void sqdem_adj_destroy(sqdem_adj* adj);
const char* sqdem_adj_last_error(sqdem_adj* adj);
/* Scene of the window: n bodies (kind, shape5 = rx ry rz eps1 eps2, wall axis/sense pairs,
 * material ids, sphere flags, state37 rows) and npairs interaction records.  Wall-wall pairs
 * are dropped, wall pairs ordered (wall, particle). */
sqdem_status sqdem_adj_load(sqdem_adj* adj, int n, const int* kind, const double* shape5, const int* wall_axis_sense,
                            const int* mat, const int* isSphere, const double* state37, long npairs,
                            const double* intr57, double dt, const double* gravity3, double damping);
/* Materials (at least as many as the bodies use): Kn, Ks, frictionAngle. */
sqdem_status sqdem_adj_set_materials(sqdem_adj* adj, int nmat, const double* Kn, const double* Ks,
                                     const double* frictionAngle);
/* Exponents of every body (n x 2; walls ignored). */
sqdem_status sqdem_adj_set_eps(sqdem_adj* adj, const double* eps2);
/* Run the window: nsteps steps, state checkpointed every checkpoint_every steps.  wF3, wX3:
 * n x 3 loss weights (NULL = 0).  Returns the loss and a 64-bit signature of every branch
 * taken (equal signatures: the same branches). */
sqdem_status sqdem_adj_forward(sqdem_adj* adj, int nsteps, int checkpoint_every, const double* wF3,
                               const double* wX3, double* loss, unsigned long long* signature);
/* Gradient of the last forward run's loss: dL/deps (n x 2), dL/dKn, dL/dKs, dL/dmu (per
 * material).  Recomputes each segment from its checkpoint; SQDEM_ERR_NUMERIC if a replay did
 * not reproduce its forward branch. */
sqdem_status sqdem_adj_backward(sqdem_adj* adj, double* dL_deps, double* dL_dKn, double* dL_dKs, double* dL_dmu);
/* State after the window: n x 16 (pos ori(w,x,y,z) vel angVel angMom). */
sqdem_status sqdem_adj_get_state(sqdem_adj* adj, double* out16);
long sqdem_adj_num_pairs(sqdem_adj* adj);
/* Pairs after the window, 16 doubles each: id1 id2 hasGeom depth contactAngle2 normal3
 * shearForce3, then the force on id1 in the last step (3) and whether it was applied. */
sqdem_status sqdem_adj_get_pairs(sqdem_adj* adj, double* out16);
/* Forward kernel of the pairs: cooperative = 1 (default) shares each Disfunction evaluation
 * among six lanes (the independent pow calls of each level on separate lanes), 0 runs the
 * pair on one thread.  Both give bitwise the same results. */
sqdem_status sqdem_adj_set_forward(sqdem_adj* adj, int cooperative);
/* Shape of the pairs' reverse-step kernel, which replays each pair's narrowphase and law in
 * dual numbers: 0 one thread per pair with all seventeen tangent components, 1 three lanes with
 * six each, 2 two lanes with nine, 3 (default) six lanes with three.  Every shape gives bitwise
 * the same gradients. */
sqdem_status sqdem_adj_set_replay(sqdem_adj* adj, int shape);
/* Resident blocks per SM of the grouped reverse-step kernels (grid-stride over the pairs;
 * default 1): each lane keeps its replayed state in local memory (a few KB), and bounding the
 * resident lanes keeps that state in L2 instead of DRAM.  0: one block per group of pairs.
 * Gradients are bitwise the same for every value. */
sqdem_status sqdem_adj_set_replay_blocks(sqdem_adj* adj, int blocks_per_sm);
/* Branch tape of the forward runs: 0 (default) evaluates every decision; 1 records the outcome
 * of every decision at which the step map jumps or kinks (the Levenberg-Marquardt path, the
 * narrowphase restarts, the bounding-sphere and contact gates, the shear reset, the Coulomb
 * cap, the local damping's signs) in each following forward run; 2 makes the following forward
 * runs take the recorded outcomes (over at most as many steps as the recorded run), so that a
 * run with perturbed parameters stays on the recorded branches and central differences are
 * those of one smooth branch.  The reverse pass always evaluates its decisions: gradients are
 * those of the recorded (natural) run.  SQDEM_ERR_STATE for 2 without a recording; a new scene
 * drops the recording. */
sqdem_status sqdem_adj_set_branches(sqdem_adj* adj, int mode);
/* Of the last forward run: decisions taken, forced decisions whose natural outcome differed,
 * decisions beyond the tape's 224 per pair and step (evaluated, not forced), steps recorded,
 * and (forced runs) pair steps whose surface evaluations saw other signs of the local
 * directions' components than the recorded run: the superquadric's support point has no
 * derivative where such a component crosses 0, so no branch can be forced there. */
sqdem_status sqdem_adj_branch_report(sqdem_adj* adj, double* out5);
/* replay mismatches, Disfunction evaluations and LM calls of the forward run, pairs replayed,
 * forward ms, backward ms, steps, checkpoint interval */
sqdem_status sqdem_adj_report(sqdem_adj* adj, double* out8);

#ifdef __cplusplus
}
#endif
#endif
