/*
 * dnl_gpu.h -- C ABI of libdnlgpu.so, the GB300 (sm_103a) FP64 implementation of DynELA's
 * explicit-dynamics step: element internal forces with J2 radial return, deterministic nodal
 * assembly, critical time step and Chung-Hulbert nodal update.
 *
 * Plain C types only.  Every function returns a status code (DNL_OK = 0).  One handle owns all
 * device memory of one mesh and a CUDA stream of its own; a handle is used by one host thread at a
 * time.  Host arrays passed in are borrowed for the duration of the call and copied.
 *
 * Reference interfaces replaced (pantale/ReDynELA, paths under Sources/Libraries/):
 *   dnl_internal_forces  -> Domain::computeInternalForces()        finiteElement/Domain.h:103,
 *                           Domain.C:130-738 (a new strategy next to the OpenMP cases 0-7) and the
 *                           Element::computeInternalForces/computeStress it calls, Element.C:164-403
 *   dnl_create           -> Domain::initSolve()                     Domain.C:1018-1226
 *   dnl_step / dnl_run   -> ExplicitSolverCH::solve(Real upTime)     ExplicitSolverCH.C:115-278,
 *                           the virtual Solver::solve of finiteElement/Solver.h:126
 *   dnl_time_step        -> Solver::computeTimeStep(Boolean)        Solver.C:220-267
 *   dnl_get/set_state    -> the Node / NodalField / IntegrationPoint members the reference keeps on
 *                           the host (Node.h:66-171, NodalField.h:36-97, IntegrationPoint.h:68-75)
 */
#ifndef DNL_GPU_H
#define DNL_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------------- statuses */
enum dnl_status {
  DNL_OK = 0,
  DNL_ERR_NEG_DETJ = 1,      /* negative Jacobian determinant (Element2D.C:101-109) */
  DNL_ERR_RR_NOCONV = 2,     /* radial return > 2000 iterations (Element.C:327-330) */
  DNL_ERR_JACOBI_NOCONV = 3, /* polar decomposition, 29 Jacobi sweeps (Tensor2.C:1257-1258) */
  DNL_ERR_PULSE_NOCONV = 4,  /* power iteration > 1000 iterations (Domain.C:936-939) */
  DNL_ERR_DT = 5,            /* time step not positive or not finite */
  DNL_ERR_ARG = 6,           /* invalid argument */
  DNL_ERR_CUDA = 7,          /* CUDA runtime error; dnl_error_string() has the detail */
  DNL_ERR_SINGULAR = 8,      /* singular element Jacobian (Matrix.C:1680-1690) */
  DNL_ERR_TIMEOUT = 9        /* a bounded device-side wait ran out */
};

/* element types */
#define DNL_ELQUA4NAX 0 /* ElQua4nAx: 4-node axisymmetric quad, 2x2 Gauss points */
#define DNL_ELHEX8N3D 1 /* ElHex8n3D: 8-node hexahedron, 2x2x2 Gauss points */
#define DNL_ELQUA4N2D 2 /* ElQua4n2D: 4-node plane-strain quad, 2x2 Gauss points (ElementPlane) */
#define DNL_ELTET4N3D 3 /* ElTet4n3D: 4-node tetrahedron, 1 Gauss point */
#define DNL_ELTET10N3D 4 /* ElTet10n3D: 10-node tetrahedron, 4 Gauss points (the reference's tables) */
/* Not a reference element: ElHex8n3D's geometry integrated at its centre only, with
 * Flanagan-Belytschko viscous hourglass control (dnl_set_hourglass) and a Courant length of
 * volume / largest face area.  Courant time step only. */
#define DNL_ELHEX8N3D_1PT 5

/* time-step methods (Solver::setTimeStepMethod, Solver.C:312-321) */
#define DNL_COURANT 0
#define DNL_PULSE 1

/* boundary-condition kinds */
#define DNL_BC_RESTRAIN 0 /* BoundaryRestrain: val[i] == 1 restrains component i */
#define DNL_BC_SPEED 1    /* BoundarySpeed (constant): val[i] != 0 imposes velocity val[i] */

/* handle flags */
#define DNL_FLAG_STEP_TENSORS 1 /* keep each step's dEps and R per integration point */

typedef struct dnl_handle dnl_handle;

/* Mesh and boundary conditions (Structure::createNode/createElement, attachInitialBC,
 * attachConstantBC).  Node and element order is the reference's Id order. */
typedef struct {
  int etype;            /* DNL_ELQUA4NAX, DNL_ELHEX8N3D, DNL_ELQUA4N2D, DNL_ELTET4N3D, DNL_ELTET10N3D,
                           DNL_ELHEX8N3D_1PT */
  int num_nodes;        /* N */
  int num_elements;     /* E */
  const double *coords; /* N*3, node-major (x, y, z) like Node::coords */
  const int *conn;      /* E*nen, 0-based node indices, reference local node order */
  double v0[3];         /* initial speed of every node (BoundarySpeed::applyInitial_V0) */
  int num_bc;           /* constant BC groups, applied in this order */
  const int *bc_kind;   /* num_bc: DNL_BC_RESTRAIN or DNL_BC_SPEED */
  const double *bc_val; /* num_bc*3 */
  const int *bc_start;  /* num_bc+1 offsets into bc_nodes */
  const int *bc_nodes;  /* node indices of each group */
} dnl_mesh_desc;

/* Material + IsoHardElastoplastic: sigma_y = A + B * evp^n (IsoHardElastoplastic.C:171-184) */
typedef struct {
  double young, poisson, density;
  double A, B, n;
} dnl_material;

/* ExplicitSolverCH settings (setTimes, setDissipation, setTimeStepSafetyFactor,
 * setComputeTimeStepFrequency, setTimeStepMethod) */
typedef struct {
  double end_time;     /* solver end time; the run starts at 0 */
  double rho_b;        /* spectral radius, reference default 0.8182 */
  double safety;       /* time-step safety factor, default 0.9 */
  int frequency;       /* recompute the critical time step every `frequency` increments (10) */
  int method;          /* DNL_COURANT or DNL_PULSE */
  int flags;           /* DNL_FLAG_* */
} dnl_solver_params;

/* Host-side view of the state.  NULL members are skipped.  Tensors are full 3x3 row-major per
 * integration point, (E, nip, 9), like Tensor2; they are stored symmetric on the device. */
typedef struct {
  double *coords;  /* N*3 current coordinates */
  double *du;      /* N*3 Current delta_disp */
  double *v;       /* N*3 Current mat_speed */
  double *a;       /* N*3 Current dmat_speed */
  double *disp;    /* N*3 Current disp */
  double *S;       /* E*nip*9 deviatoric stress */
  double *Eps;     /* E*nip*9 strain */
  double *EpsPlas; /* E*nip*9 plastic strain */
  double *p;       /* E*nip pressure */
  double *evp;     /* E*nip cumulated plastic strain */
  double *Sig;     /* E*nip*9 stress S + p I (read only) */
  double *mass;    /* N lumped nodal mass (read only) */
} dnl_state_view;

/* Time integration scalars (Solver members) */
typedef struct {
  double time;          /* Domain::currentTime */
  double time_step;     /* Solver::timeStep */
  double computed_step; /* Solver::computedTimeStep */
  double kinetic;       /* Domain::getTotalKineticEnergy() of the last step */
  long long increment;  /* Solver::increment */
  int done;             /* 1 once the end time is reached */
  int status;           /* first error recorded on the device */
  int bad_element;      /* element of that error, or -1 */
} dnl_time_info;

/* ------------------------------------------------------------------------------ single mesh */
/* Domain::initSolve (Domain.C:1018-1226): uploads the mesh, sets evp = 1e-10
 * (IntegrationPoint.C:117), applies the initial speed and computes the reference configuration's
 * shape-function derivatives. */
int dnl_create(const dnl_mesh_desc *mesh, const dnl_material *mat, const dnl_solver_params *sp,
               dnl_handle **out);
/* Structure::setDefaultElement + Structure::createElement (Structure.C:204-256, 1032-1036) for a
 * further element type in the same domain, which Domain::initSolve accepts within one family
 * (Domain.C:1042-1060): num_elements elements of etype, conn (E*nen, node indices) in the
 * handle's node numbering, numbered after the elements already there.  Before dnl_prologue or the
 * first step and before dnl_set_materials (which then takes one material per element of every
 * group); 3D reference elements (ElHex8n3D, ElTet4n3D, ElTet10n3D), ElHex8n3D with the Pulse time
 * step only.  Integration-point arrays of dnl_get/set_state, dnl_get_step_tensors, the results
 * files, the forward-mode sensitivities and the reverse-mode adjoint then cover every group in
 * element order.  DNL_ERR_ARG after several materials or another hardening law were set, and on a
 * batch's union mesh (dnl_batch_handle). */
int dnl_add_elements(dnl_handle *h, int etype, int num_elements, const int *conn);
int dnl_destroy(dnl_handle *h);
/* DNL_ELHEX8N3D_1PT: the viscous hourglass coefficient (default 0.05): the force resisting the
 * hourglass modes is a_h = coefficient rho c V^(2/3) / 4 times the mode's velocity.  The viscosity
 * acts on the Chung-Hulbert predicted velocity; its rate 16 coefficient c / V^(1/3) times the
 * Courant step must stay well below 1 (0.1 diverges on a Taylor bar at safety 0.9). */
int dnl_set_hourglass(dnl_handle *h, double coefficient);

int dnl_set_state(dnl_handle *h, const dnl_state_view *s);
int dnl_get_state(dnl_handle *h, dnl_state_view *s);
/* dEps and R of the last element pass, (E, nip, 9) (every group's points in element order on a
 * domain of several element types); needs DNL_FLAG_STEP_TENSORS */
int dnl_get_step_tensors(dnl_handle *h, double *dEps, double *R);

/* The drop-in of Domain::computeInternalForces(): one pass of the element loop (kinematics,
 * polar decomposition, radial return, RFI rotation, B^T sigma) and the assembly of Fint, with the
 * reference's side effects on the integration-point state.  coords / du (N*3, may be NULL to keep
 * the device copies) are the current coordinates and Current delta_disp; dt is Solver::timeStep;
 * fint (dim*N, index Id*dim+j, may be NULL) receives Domain::Fint. */
int dnl_internal_forces(dnl_handle *h, const double *coords, const double *du, double dt,
                        double *fint);

/* ExplicitSolverCH::solve prologue (ExplicitSolverCH.C:131-172): internal matrices, lumped mass,
 * one internal-force pass, computeTimeStep(True).  dnl_step/dnl_run call it when needed. */
int dnl_prologue(dnl_handle *h);
/* up to nsteps passes of the ExplicitSolverCH loop, all on the device; stops at the end time */
int dnl_step(dnl_handle *h, int nsteps, int *steps_done);
/* dnl_set_state(in) + dnl_step(nsteps) + dnl_get_state(out) in one call, with the same results
 * (the ExplicitSolverCH::solve loop, ExplicitSolverCH.C:115-278, between the Node field copies),
 * for a host that owns the nodal state between steps: the non-NULL nodal fields of `in` (coords,
 * du, v, a, disp; N*3 each) are uploaded and those of `out` downloaded after the last step
 * (integration-point fields and mass: DNL_ERR_ARG).  v, a and disp travel on a second stream while
 * the first element pass runs, and the download overlaps the next time step's computation
 * (page-locked host buffers keep the copies asynchronous).  in or out may be NULL. */
int dnl_step_host(dnl_handle *h, const dnl_state_view *in, int nsteps, dnl_state_view *out, int *steps_done);
/* the whole run to end_time */
int dnl_run(dnl_handle *h, int *steps_done);
/* nsteps steps captured once into a CUDA graph and replayed (same results as dnl_step);
 * Courant time step only (the Pulse power iteration checks convergence on the host) */
int dnl_step_graph(dnl_handle *h, int nsteps, int *steps_done);
int dnl_time_step(dnl_handle *h, double *dt);
int dnl_dt(dnl_handle *h, double *dt); /* the same as dnl_time_step */
int dnl_get_time_info(dnl_handle *h, dnl_time_info *info);
/* nodal internal forces of the last element pass, dim*N */
int dnl_get_fint(dnl_handle *h, double *fint);

/* ------------------------------------------------------------------------------ batches */
/* Many independent meshes (same element type) advanced together: each keeps its own material,
 * time step, increment counter and end time (each instance is one ExplicitSolverCH::solve of its
 * own Domain); every kernel of a step is launched once for all instances.  dnl_batch_prologue,
 * _step, _step_graph and _autotune need ElQua4nAx instances with the Courant time step (an even
 * recomputation frequency) and return DNL_ERR_ARG otherwise; dnl_batch_sens_run (sensitivities,
 * with a step schedule) takes any.  No counterpart in the reference, which solves one domain at a
 * time (Structure::solve, Structure.C:809-897). */
typedef struct dnl_batch dnl_batch;
int dnl_batch_create(int count, const dnl_mesh_desc *meshes, const dnl_material *mats,
                     const dnl_solver_params *params, dnl_batch **out);
int dnl_batch_destroy(dnl_batch *b);
int dnl_batch_prologue(dnl_batch *b);
/* nsteps increments of every unfinished instance; *active = instances not yet at their end time */
int dnl_batch_step(dnl_batch *b, int nsteps, int *active);
/* the same, captured once into a CUDA graph per (nsteps, phase) and replayed */
int dnl_batch_step_graph(dnl_batch *b, int nsteps, int *active);
/* capture (without running) the graph dnl_batch_step_graph(b, nsteps) replays from the current
 * increment; DNL_ERR_ARG when the handle's graph cache (8 graphs) is full */
int dnl_batch_graph_capture(dnl_batch *b, int nsteps);
/* How a batched step is launched: DNL_BATCH_LAUNCHES, the sequence of kernels of the single-mesh
 * step (time logic, boundary conditions, element pass, nodal update, Courant reduction), each once
 * for all instances; DNL_BATCH_PERSISTENT, one persistent cooperative kernel per step running the
 * same phases separated by grid-wide barriers (bounded waits: DNL_ERR_TIMEOUT if one runs out).
 * Results are bit for bit the same either way. */
#define DNL_BATCH_LAUNCHES 0
#define DNL_BATCH_PERSISTENT 1
int dnl_batch_set_mode(dnl_batch *b, int mode);
/* time live steps of both modes with 64, 128 and 256 threads per element-pass block (one untimed
 * step each, then steps_per_candidate rounds of one step per candidate in turn, so 6 * (1 +
 * steps_per_candidate) increments in all); keep the fastest (*block: its block size;
 * dnl_batch_get_tuning gives both) */
int dnl_batch_autotune(dnl_batch *b, int steps_per_candidate, int *block);
int dnl_batch_get_tuning(dnl_batch *b, int *mode, int *block);
int dnl_batch_set_block(dnl_batch *b, int block);
int dnl_batch_time_info(dnl_batch *b, int instance, dnl_time_info *info);
int dnl_batch_get_coords(dnl_batch *b, int instance, double *coords);
int dnl_batch_get_fint(dnl_batch *b, int instance, double *fint);
int dnl_batch_sizes(dnl_batch *b, int *elements, int *nodes);
/* the handle holding the union mesh (profiling, timer marks, stream) -- owned by the batch */
int dnl_batch_handle(dnl_batch *b, dnl_handle **h);

/* ------------------------------------------------------------- no device allocation */
/* Internal forces for callers that cannot allocate device memory: a host application or framework
 * whose memory manager owns every device byte and forbids libraries their own cudaMalloc, or a
 * process whose device-memory budget is fixed before the solver starts.  No counterpart in the
 * reference (its element loop runs on host objects).
 *
 * The computation of dnl_internal_forces, without a handle: the caller passes every input and
 * output in device memory, and the per-element force scratch (num_elements * nen * dim doubles) is
 * a fixed array inside the library, at most DNL_STATIC_MAX_ELEMENT_DOFS doubles (8 MiB; e.g.
 * 43,690 hex8, 65,536 Tet4 or 131,072 axisymmetric elements); larger meshes are rejected with
 * DNL_ERR_ARG.  Every GPU that loads the library holds that array until the process exits.  The
 * first call on a device looks up the array's device address (once per device, under a lock); make
 * that first call before any stream capture.  All calls share the array, which keeps the last
 * call's contents: calls whose GPU work overlaps race and must be serialised by the caller.  The
 * function synchronises `stream` to read the error word.  It calls no cudaMalloc, cudaFree or
 * allocating library routine.
 *
 * Accepted element types: DNL_ELQUA4NAX, DNL_ELQUA4N2D, DNL_ELHEX8N3D, DNL_ELTET4N3D,
 * DNL_ELTET10N3D (DNL_ELHEX8N3D_1PT needs nodal velocities and is rejected).
 * On a non-zero status (e.g. DNL_ERR_NEG_DETJ with *bad_element the first failing element) the
 * pass has still run over every element: fint and ip then hold that failed pass's values, where
 * dnl_internal_forces leaves its fint output untouched. */
#define DNL_STATIC_MAX_ELEMENT_DOFS (1 << 20)
typedef struct {
  int etype, num_nodes, num_elements;
  const int *conn;       /* [nen][E], node indices (component-major) */
  const int *node_start; /* N+1 offsets into node_entry */
  const int *node_entry; /* e*nen + k for each element touching the node, ascending e */
  const double *coords;  /* [3][N] current coordinates */
  const double *du;      /* [3][N] Current delta_disp */
  double *ip;            /* integration-point state, updated in place: [ncomp][E*nip], point
                            e*nip + q at column e*nip + q, components in this order:
                              S[ns] | Eps[ns] | EpsPlas[ns] | p | evp | evp^n
                            each tensor as its ns symmetric components,
                              ns = 4 (xx yy zz xy) for DNL_ELQUA4NAX and DNL_ELQUA4N2D,
                              ns = 6 (xx yy zz xy xz yz) for DNL_ELHEX8N3D, DNL_ELTET4N3D and
                                   DNL_ELTET10N3D,
                            so ncomp = 3 ns + 3 = 15 (quads) or 21 (3D); nip = 4 (quads, Tet10),
                            8 (hex8), 1 (Tet4).  evp^n is the cached power-law term (pow(evp, n)
                            for the material's n; evp starts at 1e-10) */
  double *fint;          /* out: N*dim, index n*dim + j */
  dnl_material mat;
} dnl_static_args;
int dnl_internal_forces_static(const dnl_static_args *args, void *stream, int *bad_element);

/* Back to the state dnl_create left: time 0, initial coordinates, velocity v0 on both nodal
 * fields, zero stresses and strains, evp = 1e-10 (IntegrationPoint.C:117); optionally with a new
 * material and initial velocity (NULL keeps the current ones).  The mesh, boundary conditions,
 * solver settings and device allocations stay; captured graphs are dropped.  For loops over
 * parameter sets (optimisation, sensitivities).  No counterpart in the reference, which rebuilds
 * the Structure from the .dyn deck. */
int dnl_reset(dnl_handle *h, const dnl_material *mat, const double *v0);

/* ------------------------------------------------------- materials and hardening laws */
/* The isotropic hardening attached to a Material (Material::setHardening): */
#define DNL_HARD_POWER 0   /* IsoHardElastoplastic: sigma_y = A + B evp^n, params = A, B, n
                              (IsoHardElastoplastic.C:171-184) */
#define DNL_HARD_ELASTIC 1 /* none attached: the material never yields (Material::isYield,
                              Material.C:366-371) */
#define DNL_HARD_TABULAR 2 /* IsoHardElastoplasticTabular: a DiscreteFunction of evp, points in
                              ascending abscissa (IsoHardElastoplasticTabular.C:103-116,
                              DiscreteFunction.C:169-201, 274-297) */
#define DNL_HARD_METAFOR 3 /* IsoHardMetafor: params = P1..P8, sigma_y = (P2-P1)(1-exp(-P3 evp))
                              + P4 evp^P5 + P1 (1 + P6 evp)^P7 + P8 evp (IsoHardMetafor.C:132-153) */
typedef struct {
  double young, poisson, density;
  int law;                        /* DNL_HARD_* */
  double params[8];
  int npoints;                    /* DNL_HARD_TABULAR */
  const double *table_x, *table_y;
} dnl_material_law;
/* Several materials in one mesh (Structure::attachMaterialToElements per ElementSet) and any of
 * the hardening laws: element e gets mats[elem_material[e]] (elem_material NULL: one material for
 * all).  As Domain::initSolve, each node's density is that of the last element holding it and the
 * Courant sound speed of an element averages those densities; the Pulse power iteration forms
 * each element's K x with its own material's Hooke matrix (Element3D.C:242-333).  Before the
 * prologue.  Sensitivity runs need one power-law material. */
int dnl_set_materials(dnl_handle *h, int nmat, const dnl_material_law *mats, const int *elem_material);

/* -------------------------------------------------------------- results / restart files */
/* The reference's binary results file (Structure::writeData, Structure.C:936-952, through
 * io_Data::structure_write, io_Data.C:486-506): version header, time, per node the coordinates
 * and the Current NodalField, per integration point p, evp, S, Sig, Eps, dEps, EpsPlas (each
 * element's own points, elements in the domain's order, on a domain of several element types).
 * Writing needs the last step's strain increments: a handle created with DNL_FLAG_STEP_TENSORS
 * (DNL_ERR_ARG otherwise). */
int dnl_write_results(dnl_handle *h, const char *path);
/* Load such a file into the handle (same mesh) and continue from its time: coordinates, Current
 * nodal fields and integration-point state are replaced, the lumped mass stays that of the initial
 * mesh, and the time step is recomputed on the loaded state (Solver::computeTimeStep(True)). */
int dnl_read_results(dnl_handle *h, const char *path);

/* ------------------------------------------------------------------- sensitivities */
/* Derivatives of a run's final nodal coordinates with respect to four parameters: the hardening
 * law's A, B, n (sigma_y = A + B evp^n, IsoHardElastoplastic.C:171-184) and the magnitude |v0| of
 * the initial velocity v0 = |v0| u (BoundarySpeed::applyInitial_V0, Boundary.C:378-385).  The run
 * is ExplicitSolverCH::solve's loop (ExplicitSolverCH.C:179-274) with the step sizes taken from a
 * caller's schedule (a parameter-independent dt sequence) instead of Solver::computeTimeStep, from
 * the handle's initial state (no step taken yet); the end time is not applied.  Computed in
 * forward mode (four tangent copies of the state advanced with it), which for four parameters
 * stores no trajectory.  Every element type; one power-law material.  No counterpart in the
 * reference, which has no derivatives. */
#define DNL_SENS_NPARAM 4 /* A, B, n, |v0| */
/* nsteps steps with step sizes dts[0..nsteps); coords (3N, node-major, may be NULL) receives the
 * final coordinates, dcoords (4 x 3N, may be NULL) their derivatives, dcoords[p*3N + 3n + j] */
int dnl_sens_run(dnl_handle *h, int nsteps, const double *dts, double *coords, double *dcoords);
/* step-size schedule used by dnl_adjoint */
int dnl_set_dt_schedule(dnl_handle *h, const double *dts, int nsteps);
/* The gradient of a loss L(x_final) in reverse mode: grad[p] = sum dL/dx . dx/dp for p = A, B, n,
 * |v0|, given dL/dx_final (3N, node-major), over the schedule set by dnl_set_dt_schedule, from the
 * handle's initial state (no step taken yet, as dnl_sens_run).  One forward sweep stores the state
 * every ckpt_stride steps (ckpt_stride = 0: ceil(sqrt(nsteps))); the reverse sweep restores each
 * segment from its checkpoint, runs it again storing its steps' states (and, within
 * dnl_set_adjoint_record_budget, their per-point records), and undoes its steps in reverse order
 * through the adjoints of the nodal update, the element pass (kinematics, polar decomposition, J2
 * return, RFI rotation, forces) and the assembly.  Memory: ceil(nsteps / ckpt_stride) checkpoints
 * plus ckpt_stride step states (dnl_adjoint_stats), so O(sqrt(nsteps)) with the default; cost:
 * about three forward runs.  The same linearisation as the forward mode
 * (dnl_sens_run), so the two gradients agree to rounding.  One power-law material; every element
 * type but DNL_ELHEX8N3D_1PT.  The handle is back at its initial state afterwards.  No counterpart
 * in the reference, which has no derivatives. */
int dnl_adjoint(dnl_handle *h, const double *dL_dx, double *grad, int ckpt_stride);
/* dnl_adjoint in two calls, for a caller that needs the final coordinates to form dL/dx: the
 * forward sweep (the scheduled run from the initial state with its checkpoints; coords, 3N
 * node-major, may be NULL, receives the final coordinates; the handle is left at the final state),
 * then the reverse sweep over those checkpoints (the handle is back at its initial state after).
 * dnl_adjoint_backward without a preceding forward sweep returns DNL_ERR_ARG. */
int dnl_adjoint_forward(dnl_handle *h, int ckpt_stride, double *coords);
int dnl_adjoint_backward(dnl_handle *h, const double *dL_dx, double *grad);
typedef struct {
  int nsteps;                  /* steps of the schedule */
  int stride;                  /* steps per checkpoint segment */
  int checkpoints;             /* states stored by the forward sweep */
  long long recomputed_steps;  /* steps run again by the reverse sweep */
  long long bytes;             /* device memory of the adjoint (checkpoints, step states, adjoints) */
  long long checkpoint_bytes;  /* of which the checkpoints */
  long long record_bytes;      /* of which one segment's step states */
  long long kept_record_bytes; /* of which one segment's per-point records (0: regenerated) */
} dnl_adjoint_info;
/* figures of the last dnl_adjoint on this handle */
int dnl_adjoint_stats(dnl_handle *h, dnl_adjoint_info *info);
/* Device memory the reverse sweep may spend (per handle) on keeping a segment's per-point records,
 * which its recomputation writes, so that undoing a step does not run the element pass again:
 * used when ckpt_stride x the records of one step fit (default 2 GiB; 0: every record is
 * regenerated).  Gradients are the same bit for bit either way.  Applies to sweeps started after
 * the call.  No counterpart in the reference. */
int dnl_set_adjoint_record_budget(unsigned long long bytes);
/* The scheduled run alone (no derivatives): nsteps steps of sizes dts from the handle's initial
 * state; coords (3N, node-major, may be NULL) receives the final coordinates.  The primal of
 * dnl_sens_run and of dnl_adjoint, bit for bit. */
int dnl_run_schedule(dnl_handle *h, int nsteps, const double *dts, double *coords);
/* The same for every instance of a batch at once, all with the schedule dts, from the batch's
 * initial state; coords (3 x total nodes) and dcoords (4 x 3 x total nodes) in the union's node
 * order (instance after instance, see dnl_batch_sizes).  A batch created for this may hold
 * instances of either element type with either time-step method (the schedule replaces it). */
int dnl_batch_sens_run(dnl_batch *b, int nsteps, const double *dts, double *coords, double *dcoords);
/* every instance back to its initial state (as dnl_batch_create left it), device buffers kept */
int dnl_batch_reset(dnl_batch *b);
/* the state of a single-mesh handle of the same mesh (coordinates, Current nodal field,
 * integration-point state; evp^n recomputed with each instance's n) copied into every instance,
 * on the device; the time records are kept.  For starting a batch from a state one run reached,
 * e.g. timing the plastic phase of a long schedule.  DNL_ERR_ARG unless every instance has the
 * handle's element type and sizes. */
int dnl_batch_broadcast_state(dnl_batch *b, dnl_handle *src);

/* -------------------------------------------------------------------------- measurement */
/* Per-kernel device time: between dnl_profile_begin and dnl_profile_end the library brackets each
 * of its launches on the handle's stream with CUDA events; dnl_profile_end synchronises and returns
 * the summed milliseconds and launch counts per kernel class. */
#define DNL_PROF_ELEM 0    /* k_elem: element pass (kinematics, stress, forces) */
#define DNL_PROF_NODE 1    /* k_node / k_gather: assembly and nodal update */
#define DNL_PROF_PULSE 2   /* Pulse power-iteration kernels */
#define DNL_PROF_COURANT 3 /* Courant length reduction */
#define DNL_PROF_OTHER 4   /* time-step logic, boundary conditions */
#define DNL_PROF_TANGENT 5 /* sensitivity run: tangent element pass (its nodal pass counts as NODE) */
#define DNL_PROF_KINDS 6
int dnl_profile_begin(dnl_handle *h);
int dnl_profile_end(dnl_handle *h, double *ms, long long *launches);
/* the handle's CUDA stream (a cudaStream_t), e.g. to record timing events around calls */
int dnl_get_stream(dnl_handle *h, void **stream);

/* Device-time marks on the handle's stream: dnl_timer_mark records CUDA event `slot` (0..7);
 * dnl_timer_elapsed waits for `to` and returns the milliseconds between the two marks. */
int dnl_timer_mark(dnl_handle *h, int slot);
int dnl_timer_elapsed(dnl_handle *h, int from, int to, double *ms);
/* NVTX ranges around a caller's region (profilers can restrict capture to it) */
int dnl_range_push(const char *name);
int dnl_range_pop(void);
/* FP64 fused multiply-add throughput of the current device, measured by a dependent-chain kernel
 * over all SMs (TFLOP/s, 2 flops per DFMA) */
int dnl_measure_fp64_peak(double *tflops);
/* Limits of the three bounded loops of the step, for exercising the non-convergence statuses:
 * Jacobi passes of the polar decomposition (0..29, default 29, Tensor2.C:1169-1258 ->
 * DNL_ERR_JACOBI_NOCONV), Newton iterations of the radial return (0..2000, default 2000,
 * Element.C:327-330 -> DNL_ERR_RR_NOCONV) and Pulse power iterations (1..1000, default 1000,
 * Domain.C:936-939 -> DNL_ERR_PULSE_NOCONV).  A negative value restores the reference's default.
 * Process-wide; the two element-pass limits are device constants of the current device.  Change
 * them only between runs (no call of the library in flight).  No counterpart in the reference,
 * whose limits are literals. */
int dnl_set_iteration_caps(int rotations, int newton, int power);
/* Stopping tests of the element pass's two iterations: the polar decomposition stops once every
 * off-diagonal |C_pq| < polar (Tensor2.C:1180, default 1e-9) and the radial return once
 * |f / sigma_y| <= radial (Element.C:315, default 1e-8).  A negative value restores the reference's
 * default; 0 or >= 1 is refused.  Tighter tolerances move results away from the reference's, which
 * the parity tests hold at the defaults; they exist to check derivatives (dnl_sens_run,
 * dnl_adjoint) against difference quotients of the run: with the reference's tolerances a
 * parameter change of 1e-6 relative can add or remove an iteration somewhere, a jump in the run's
 * map of the tolerance's order that a difference quotient divides by h.  Process-wide device
 * constants of the current device; change them only between runs.  No counterpart in the
 * reference, whose tolerances are literals. */
int dnl_set_stop_tolerances(double polar, double radial);
/* Self-check of the element and nodal kernels' division helpers on the current device: for each
 * i < n, out[i] = the Newton-Raphson reciprocal 1/b[i] the kernels use, out[n + i] = their quotient
 * a[i]/b[i] (reciprocal + one residual correction), out[2n + i] = CUDA's IEEE 1.0/b[i] and
 * out[3n + i] = its IEEE a[i]/b[i], for comparison.  No counterpart in the reference (which
 * divides in IEEE arithmetic). */
int dnl_check_quotients(int n, const double *a, const double *b, double *out);

/* --------------------------------------------------------------------------------- misc */
/* select the CUDA device used by subsequent dnl_create calls of this thread */
int dnl_set_device(int device);
/* page-locked host memory for fast host <-> device state transfers */
int dnl_host_alloc(unsigned long long bytes, void **ptr);
int dnl_host_free(void *ptr);
const char *dnl_error_string(int status);
int dnl_device_count(int *count);
/* number of kernels this library launched (all handles), for launch accounting */
long long dnl_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif
