/*
 * sdg_gpu.h -- C ABI of the GB300 explicit DG residual-and-update path.
 *
 * This is the drop-in boundary that replaces SubrosaDG's templated
 * Solver<SimulationControl> seam (src/Solver/SolveControl.cpp:327-436), which
 * System<SimulationControl>::solve (src/Utils/SystemControl.cpp:159-195) drives.
 * A C++ host shim marshals the reference's Mesh/PhysicalModel/BoundaryCondition
 * objects into the plain arrays below and calls these entry points; the library
 * owns all device memory, the caller owns every host buffer (copied in/out).
 *
 * Conventions
 *   - Every entry point returns SDG_OK (0) or an SDG_ERR_* code and never throws.
 *     sdg_last_error(handle) (or sdg_last_error(NULL) after a failed create)
 *     returns a NUL-terminated description of the last failure.
 *   - Calls are synchronous with respect to the handle's CUDA stream unless the
 *     name ends in _async.  A handle is not thread-safe; one handle = one GPU.
 *   - All arithmetic is IEEE FP64.  Integer data are int32 connectivity.
 *   - Element blocks are ordered as the reference orders its element loops:
 *     2D: triangles then quadrangles; 3D: hexahedra
 *     (src/Solver/SpatialDiscrete.cpp:268-291).
 *   - "Volume points" are the reference's volume quadrature points
 *     (Gauss rule of order 2P, src/Solver/SimulationControl.cpp:275-278);
 *     per-point arrays are [element][point][component] in block order.
 *   - Conserved variables: rho, rho*u (d components), rho*E.
 *     Primitive variables: rho, u (d components), T (src/Solver/VariableConvertor.cpp:332-366).
 */
#ifndef SDG_GPU_H_
#define SDG_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------------------------- */
#define SDG_OK 0
#define SDG_ERR_INVALID_ARGUMENT 1 /* bad pointer, count, enum or size                                */
#define SDG_ERR_CUDA 2             /* a CUDA runtime call failed (text in sdg_last_error)           */
#define SDG_ERR_OUT_OF_MEMORY 3    /* device allocation failed                                      */
#define SDG_ERR_MESH 4             /* inconsistent mesh: a face seen more than twice, unmatched
                                      boundary face, inverted element (Adjacency.cpp:161-165)      */
#define SDG_ERR_UNSUPPORTED 5      /* configuration outside what this build implements              */
#define SDG_ERR_NONFINITE 6        /* NaN/Inf detected in the state (SystemControl.cpp:185-191)     */
#define SDG_ERR_TIMEOUT 7          /* a bounded device wait gave up                                  */
#define SDG_ERR_STATE 8            /* call out of order (e.g. step before an initial state)         */

/* ---- enumerations (values equal the reference's enum order, src/Utils/Enum.cpp) --------------- */
enum sdg_element_type { /* gmsh first-order type numbers (src/Solver/SimulationControl.cpp:26-31) */
  SDG_ELEMENT_LINE = 1,     /* DimensionEnum::D1 / MeshModelEnum::Line; its faces are points */
  SDG_ELEMENT_TRIANGLE = 2,
  SDG_ELEMENT_QUADRANGLE = 3,
  SDG_ELEMENT_TETRAHEDRON = 4, /* dense modal blocks, P = 1..5, every equation model and the artificial
                                  viscosity, and their derivatives for P = 1..3 (not of the artificial
                                  viscosity)                                                          */
  SDG_ELEMENT_HEXAHEDRON = 5
};
enum sdg_equation {                                                                    /* Enum.cpp:56-64   */
  SDG_COMPRESSIBLE_EULER = 0,
  SDG_COMPRESSIBLE_NS = 1,
  SDG_INCOMPRESSIBLE_EULER = 2, /* the weakly compressible fluid of EquationOfState WeakCompressibleFluid:  */
  SDG_INCOMPRESSIBLE_NS = 3     /* conserved (rho, rho u, rho e), p = c0^2 (rho - rho0) + 0.01 rho0 c0^2     */
};
enum sdg_convective_flux {                                                            /* Enum.cpp:107-113 */
  SDG_FLUX_CENTRAL = 0,
  SDG_FLUX_LAX_FRIEDRICHS = 1,
  SDG_FLUX_HLLC = 2,
  SDG_FLUX_ROE = 3,
  SDG_FLUX_EXACT = 4          /* incompressible models only (ConvectiveFlux.cpp:352-414)                   */
};
enum sdg_source_term { SDG_SOURCE_NONE = 0, SDG_SOURCE_BOUSSINESQ = 1 };               /* Enum.cpp:71-74   */
enum sdg_shock_capturing { SDG_SHOCK_NONE = 0, SDG_SHOCK_ARTIFICIAL_VISCOSITY = 1 };    /* Enum.cpp:76-79   */
enum sdg_viscous_flux { SDG_VISCOUS_NONE = 0, SDG_VISCOUS_BR1 = 1, SDG_VISCOUS_BR2 = 2 }; /* Enum.cpp:115-119 */
enum sdg_time_integration {                                                            /* Enum.cpp:136-140 */
  SDG_FORWARD_EULER = 0,
  SDG_HEUN_RK2 = 1,
  SDG_SSPRK3 = 2
};
enum sdg_transport_model { SDG_TRANSPORT_NONE = 0, SDG_TRANSPORT_CONSTANT = 1, SDG_TRANSPORT_SUTHERLAND = 2 };
enum sdg_boundary_condition {                                                          /* Enum.cpp:92-100 */
  SDG_BC_RIEMANN_FARFIELD = 0,
  SDG_BC_VELOCITY_INFLOW = 1,
  SDG_BC_PRESSURE_OUTFLOW = 2,
  SDG_BC_ISOTHERMAL_NONSLIP_WALL = 3,
  SDG_BC_ADIABATIC_SLIP_WALL = 4,
  SDG_BC_ADIABATIC_NONSLIP_WALL = 5,
  SDG_BC_PERIODIC = 6
};

/* ---- mesh: first-order (straight-sided) geometry in gmsh vertex order -------------------------- */
typedef struct sdg_mesh {
  int32_t dimension;                  /* 1, 2 or 3                                                  */
  int64_t node_count;
  const double* node_coordinate;      /* [node_count][3]                                            */
  const int32_t* periodic_master;     /* [node_count] node -> periodic master node (itself when not a
                                         slave), or NULL.  Replaces gmsh::getPeriodicNodes pairing
                                         (src/Mesh/Adjacency.cpp:213-328).  1D without a map: the two
                                         periodic boundary points are joined, the first one's element
                                         on the left (Adjacency.cpp:185-211).                       */
  int64_t triangle_count;
  const int32_t* triangle_node;       /* [triangle_count][3]                                        */
  int64_t quadrangle_count;
  const int32_t* quadrangle_node;     /* [quadrangle_count][4]                                      */
  int64_t hexahedron_count;
  const int32_t* hexahedron_node;     /* [hexahedron_count][8]                                      */
  int64_t boundary_count;             /* boundary elements: points (1D), lines (2D), quadrangles or
                                         triangles (3D; a triangle's fourth index is -1)             */
  const int32_t* boundary_node;       /* [boundary_count][1, 2 or 4]                                */
  const int32_t* boundary_physical;   /* [boundary_count] 1-based physical group index              */
  int32_t physical_count;
  const int32_t* physical_boundary_condition; /* [physical_count] sdg_boundary_condition per group,
                                                 as System::addBoundaryCondition sets it
                                                 (src/Utils/SystemControl.cpp:76-80)                */
  int64_t line_count;                 /* 1D: line elements, vertex 0 then vertex 1 (x increasing: the
                                         reference's point normals are -1 at local face 0 and +1 at
                                         local face 1, Geometry.cpp:102-112)                        */
  const int32_t* line_node;           /* [line_count][2]                                            */
  int64_t tetrahedron_count;          /* 3D: tetrahedra (MeshModelEnum::Tetrahedron), gmsh vertex order */
  const int32_t* tetrahedron_node;    /* [tetrahedron_count][4]                                      */
  /* Curved (high-order) geometry, as the drivers' setOrder(P) makes it and src/Mesh/ReadControl.cpp:243-256
     reads it: geometry_order q in 2..5 (0 or 1: straight-sided) and, per element, the node indices of its
     order-q Lagrange element in gmsh's node order (the corners first, equal to the vertex lists above).  The
     Jacobians and face normals are then those of the order-q map at every quadrature point
     (src/Mesh/Geometry.cpp:44-86, 102-147).  Triangles, quadrangles and hexahedra; tetrahedra stay
     straight-sided.                                                                                 */
  int32_t geometry_order;
  const int32_t* triangle_geometry_node;   /* [triangle_count][(q+1)(q+2)/2], or NULL                  */
  const int32_t* quadrangle_geometry_node; /* [quadrangle_count][(q+1)^2], or NULL                     */
  const int32_t* hexahedron_geometry_node; /* [hexahedron_count][(q+1)^3], or NULL                     */
} sdg_mesh;

/* ---- physics and numerics: the runtime form of the reference's SimulationControl -------------- */
typedef struct sdg_config {
  int32_t polynomial_order;           /* 1..5 (Enum.cpp:48-54)                                      */
  int32_t equation;                   /* sdg_equation                                               */
  int32_t convective_flux;            /* sdg_convective_flux                                        */
  int32_t viscous_flux;               /* sdg_viscous_flux (NS only)                                 */
  int32_t time_integration;           /* sdg_time_integration                                       */
  int32_t transport_model;            /* sdg_transport_model (NS only)                              */
  double specific_heat_ratio;         /* reference: constexpr 1.4 (src/Solver/PhysicalModel.cpp:45) */
  double specific_heat_constant_pressure; /* System::setThermodynamicModel (SystemControl.cpp:82-88) */
  double specific_heat_constant_volume;
  double dynamic_viscosity;           /* System::setTransportModel (SystemControl.cpp:98-103)       */
  double prandtl_number;              /* reference: constexpr 0.71 (PhysicalModel.cpp:91)           */
  /* incompressible models (System::setEquationOfState, PhysicalModel.cpp:57-78); compressible ones use the
     ideal gas with specific_heat_ratio and compressible fluxes (Central, LF, HLLC, Roe)                     */
  double reference_sound_speed;       /* c0                                                             */
  double reference_density;           /* rho0                                                           */
  int32_t source_term;                /* sdg_source_term                                                */
  double thermal_expansion_coefficient; /* Boussinesq beta (SourceTerm.cpp:35-38), gravity 1 along the last
                                           coordinate (y in 2D, z in 3D)                                   */
  double reference_temperature;       /* Boussinesq T_ref                                               */
  /* shock capturing (System::setArtificialViscosity, SystemControl.cpp:105-108): per-step Persson-Peraire
     density sensor, eps = factor * h / P ramped over [s0 - tolerance, s0 + tolerance], vertex max        */
  int32_t shock_capturing;            /* sdg_shock_capturing                                            */
  double empirical_tolerance;         /* kappa of the sensor ramp (> 0 with artificial viscosity)       */
  double artificial_viscosity_factor; /* eps0 (the reference's default 1.0)                             */
} sdg_config;

/* ---- sizes of a created problem ------------------------------------------------------------- */
typedef struct sdg_counts {
  int32_t dimension;
  int32_t conserved_variable_count;   /* d + 2                                                      */
  int32_t block_count;                /* element blocks (one per element type present)              */
  int32_t block_element_type[2];      /* sdg_element_type of each block                             */
  int64_t block_element_count[2];
  int32_t block_basis_count[2];       /* Nb per element                                             */
  int32_t block_volume_point_count[2];/* Nq per element                                             */
  int64_t element_count;              /* all blocks                                                 */
  int64_t volume_point_count;         /* sum over blocks of elements * Nq                           */
  int64_t degree_of_freedom_count;    /* sum of elements * Nb * (d+2)                               */
  int64_t interior_face_count;
  int64_t boundary_face_count;
  int32_t face_point_count;           /* Nfq per face (order 2P+1 rule)                             */
  int64_t boundary_point_count;       /* boundary_face_count * face_point_count                     */
} sdg_counts;

typedef struct sdg_handle sdg_handle;

/* Last error text for this handle (or the last failed sdg_create when handle is NULL). */
const char* sdg_last_error(const sdg_handle* handle);

/* Build the problem: adjacency and periodic pairing (Adjacency.cpp:432-495), geometry
 * (Geometry.cpp:44-169), operators, device buffers.  Replaces Mesh<SC>::readMeshElement
 * (src/Mesh/ReadControl.cpp:293-335) + Solver<SC> member construction.  device = CUDA ordinal;
 * device < 0 builds a host-only handle (adjacency, geometry, coordinates, counts; no GPU is touched
 * and every state/step entry point returns SDG_ERR_STATE). */
int sdg_create(const sdg_mesh* mesh, const sdg_config* config, int32_t device, sdg_handle** handle);
int sdg_destroy(sdg_handle* handle);
int sdg_get_counts(const sdg_handle* handle, sdg_counts* counts);

/* Physical coordinates of every volume point, [volume_point_count][3]
 * (ElementMesh::quadrature_node_coordinate_, src/Mesh/Geometry.cpp:51-58). */
int sdg_volume_point_coordinate(sdg_handle* handle, double* coordinate);
/* Physical coordinates of every boundary face point, [boundary_point_count][3], and the
 * 1-based physical group of each boundary face, [boundary_face_count]. */
int sdg_boundary_point_coordinate(sdg_handle* handle, double* coordinate, int32_t* physical);

/* Initial condition from primitive values (rho,u,T) at the volume points: conserved
 * conversion + unweighted least-squares projection, as Solver::initializeSolver does
 * (src/Solver/InitialCondition.cpp:85-104). */
int sdg_set_initial_primitive(sdg_handle* handle, const double* primitive);
/* Ghost primitive states at boundary face points, [boundary_point_count][d+2]
 * (AdjacencyElementSolver::boundary_dummy_variable_, InitialCondition.cpp:118-149). */
int sdg_set_boundary_primitive(sdg_handle* handle, const double* primitive);

/* State exchange in physical space: conserved values at the volume points,
 * [volume_point_count][d+2].  set = unweighted least-squares projection. */
int sdg_set_state_point(sdg_handle* handle, const double* conserved);
int sdg_get_state_point(sdg_handle* handle, double* conserved);
/* State exchange as modal coefficients in the reference's per-element layout
 * (variable_basis_function_coefficient_: column-major (d+2) x Nb, SolveControl.cpp:45-60),
 * concatenated per block.  Basis: the hierarchic Lobatto basis (integrated Legendre polynomials,
 * l0 = (1-x)/2, l1 = (1+x)/2, l_k = (P_k - P_{k-2}) / sqrt(2(2k-1)) for k >= 2), tensor products of it on
 * quadrangles and hexahedra (gmsh's H1Legendre family, src/Mesh/BasisFunction.cpp:46-74). */
int sdg_set_state_modal(sdg_handle* handle, const double* coefficient);
int sdg_get_state_modal(sdg_handle* handle, double* coefficient);

/* dt = min over volume points of CFL * minEdge / ((|u|+c)(P+1)^2)
 * (Solver::calculateDeltaTime, src/Solver/TimeIntegration.cpp:104-131). */
int sdg_calculate_delta_time(sdg_handle* handle, double courant_friedrichs_lewy_number, double* delta_time);

/* Advance step_count full RK steps of size delta_time (Solver::stepSolver,
 * src/Solver/TimeIntegration.cpp:326-350).  After the last step the relative error of that
 * step is available from sdg_relative_error. */
int sdg_step(sdg_handle* handle, int32_t step_count, double delta_time);
/* Same, enqueued on the handle's stream without a host synchronisation. */
int sdg_step_async(sdg_handle* handle, int32_t step_count, double delta_time);
/* One step (sdg_step with step_count 1) that also returns the new state as sdg_get_state_point does, and
 * the step's relative error when relative_error is not null (d+2 doubles).  The reference's solve loop
 * reads the state after Solver::stepSolver (src/Solver/TimeIntegration.cpp:326-350) for its views; here,
 * when `conserved` is pinned host memory (cudaHostAlloc / cudaHostRegister), the last RK stage of tensor
 * blocks writes each element's new state straight into it while the stage computes, so no transfer
 * follows the step; dense blocks, and pageable buffers, are converted and copied after the step.  The
 * captured step graph is re-captured when the buffer differs from the previous call's. */
int sdg_step_state_point(sdg_handle* handle, double delta_time, double* conserved, double* relative_error);
/* One step from a host state to a host state: conserved_in becomes the state (as sdg_set_state_point), it is
 * advanced one step (sdg_step) and the new state is written to conserved_out (as sdg_step_state_point), with
 * the step's relative error when relative_error is not null.  The input crosses to the device into a staging
 * buffer of its own (volume_point_count x (d+2) doubles, allocated on first use) on a stream of its own: read
 * in place by a narrow copy kernel when pinned, by the copy engine when pageable.
 * The _async form returns once the work is enqueued: the transfer of a call's input then runs while the
 * previous call's step computes, for a caller streaming independent states through the solver.  Both buffers
 * must stay valid and unchanged until sdg_synchronize; sdg_relative_error then gives the last call's relative
 * error.  Pinned buffers (cudaHostAlloc / cudaHostRegister) make both transfers asynchronous; with pageable
 * ones the copies are staged by the driver and the calls wait for them.  States, point values and relative
 * errors are those of sdg_set_state_point + sdg_step + sdg_get_state_point, bit for bit. */
int sdg_step_state_point_from(sdg_handle* handle, double delta_time, const double* conserved_in,
                              double* conserved_out, double* relative_error);
int sdg_step_state_point_from_async(sdg_handle* handle, double delta_time, const double* conserved_in,
                                    double* conserved_out);

/* Solver::relative_error_ of the last step: per conserved variable, the element mean of
 * mean_q |R Phi^T| (TimeIntegration.cpp:279-324).  NaN entries signal a blow-up. */
int sdg_relative_error(sdg_handle* handle, double* relative_error);

/* One spatial-residual evaluation at the current state, returned as du/dt = M^-1 R at the
 * volume points, [volume_point_count][d+2] (SpatialDiscrete.cpp:1016-1032 followed by the
 * M^-1 of TimeIntegration.cpp:196). */
int sdg_residual_point(sdg_handle* handle, double* rate);

/* Wait for all work on the handle's stream. */
int sdg_synchronize(sdg_handle* handle);

/* Diagnostic: number of CUDA kernel launches issued by this handle since creation. */
int sdg_launch_count(const sdg_handle* handle, int64_t* launch_count);

/* The handle's CUDA stream (a cudaStream_t), for callers that enqueue their own work or events on it. */
int sdg_get_stream(const sdg_handle* handle, void** stream);

/* Diagnostic kernel timing.  While enabled every launch is bracketed by CUDA events on the handle's
 * stream; sdg_kernel_time synchronises and returns, per kernel class -- 0 element stage kernels,
 * 1 interior-face flux / trace exchange, 2 boundary-face flux / exchange, 3 other (reductions,
 * conversions), 4 gradient kernels (Navier-Stokes) -- the summed device milliseconds and launch counts
 * (arrays of 5) since timing was (re-)enabled. */
int sdg_set_kernel_timing(sdg_handle* handle, int32_t enable);
int sdg_kernel_time(sdg_handle* handle, double* milliseconds, int64_t* launches);

/* Diagnostic: sustained FP64 FMA rate of the device, in GFLOP/s (2 flops per FMA), from an
 * independent-chain FMA kernel run for about `milliseconds` ms.  Used as the FP64 roofline. */
int sdg_measure_fp64_peak(int32_t device, double milliseconds, double* gflops);
/* Diagnostic: FP64 tensor-core (DMMA) rate of the device, in GFLOP/s (2 M N K flops per mma), from a
 * kernel of independent mma.sync .f64 chains of one shape run for about `milliseconds` ms.
 * shape 0: m8n8k4, 1: m16n8k4, 2: m16n8k8, 3: m16n8k16.  Compared with sdg_measure_fp64_peak it decides
 * whether the basis contractions gain anything from the tensor cores. */
int sdg_measure_dmma_peak(int32_t device, int32_t shape, double milliseconds, double* gflops);
/* Diagnostic: the device reciprocal every flux kernel uses for 1/rho and the wave-speed quotients
 * (rcp.approx.ftz.f64 estimate + two Newton-Raphson steps), applied to x[0..n) on `device`: out[i] = rcp(x[i]).
 * Host buffers.  Its accuracy is checked against IEEE 1/x by the tests: within 1 ulp for normal x whose
 * reciprocal is normal (|x| in [2^-1022, 2^1022]); the flush-to-zero estimate leaves subnormal inputs
 * and outputs outside that range (no density or pressure of a flow comes near it). */
int sdg_probe_reciprocal(int32_t device, const double* x, double* out, int64_t n);

/* Diagnostic: adjacency as canonical integer tuples, for bit-exact parity checks.
 * interior: [interior_face_count][7] = (typeL, elemL, faceL, typeR, elemR, faceR, rotation)
 * boundary: [boundary_face_count][5] = (type, elem, face, physical, boundary_condition)
 * Element indices are within their block; rows sorted lexicographically. */
int sdg_adjacency(const sdg_handle* handle, int32_t* interior, int32_t* boundary);

/* Allocation-free CFL time step.  Some callers cannot call cudaMalloc where they need a time step -- a
 * framework whose memory pool forbids raw device allocations, a real-time loop that must not allocate, a
 * host that only records work into a stream it was handed.  This entry point has no counterpart in the
 * reference.  For one element block it returns the dt that sdg_calculate_delta_time computes over that
 * block, from device arrays the caller already holds, and allocates nothing:
 *   state_point   device [point_count][dimension+2] conserved values at the block's volume points
 *   minimum_edge  device [point_count / points_per_element] shortest edge per element (minEdge quality)
 *   points_per_element  volume points per element of the block; point_count must be a multiple of it
 *   dimension     1, 2 or 3
 *   specific_heat_ratio  gamma of the ideal gas (> 1; ignored when reference_sound_speed > 0)
 *   reference_sound_speed  0 for the compressible models (sound speed sqrt(gamma p / rho)); the constant c0
 *                 of the incompressible models (sdg_config.reference_sound_speed) otherwise
 *   delta_time    device pointer to one double that receives dt (overwritten by every call)
 *   stream        cudaStream_t to enqueue on (NULL: the legacy default stream); the result is ready
 *                 when the stream reaches that point
 * A mesh of several blocks (triangles and quadrangles) needs one call per block, with that block's points,
 * minEdge and points_per_element, into separate doubles; dt is their minimum, which the caller takes.
 * Its scratch is a file-scope __device__ array of 131072 doubles (1 MiB) that every GPU which loads
 * the library holds until the process exits.  point_count above 33,554,432 is rejected with
 * SDG_ERR_INVALID_ARGUMENT.  The first call on a device (and in each new CUDA context of it) looks up the
 * array's device address with that device current: make that first call before any stream capture.  All
 * calls share the array, so calls that overlap on the GPU race; serialise them.  Errors:
 * SDG_ERR_INVALID_ARGUMENT, SDG_ERR_CUDA, with text in sdg_last_error(NULL). */
int sdg_delta_time_noalloc(const double* state_point, const double* minimum_edge, int64_t point_count,
                           int32_t points_per_element, int32_t dimension, int32_t polynomial_order,
                           double specific_heat_ratio, double reference_sound_speed,
                           double courant_friedrichs_lewy_number, double* delta_time, void* stream);

/* Structured mesh generators of the reference's example drivers (gmsh transfinite + periodic
 * setups in examples/periodic_2d_ceuler.cpp:63-94 and examples/periodic_3d_ceuler.cpp:60-130),
 * plus the jittered/triangle-split hybrid of the Kelvin-Helmholtz workload.  The generator owns
 * the arrays it returns; free them with sdg_mesh_free. */
typedef struct sdg_generated_mesh {
  sdg_mesh mesh;
  void* storage;                      /* owned by the library                                       */
} sdg_generated_mesh;
/* 2D [x0,x0+lx] x [y0,y0+ly], nx x ny quadrangles; jitter = fraction of h for interior nodes
 * (seeded); split_fraction = fraction of quads split into two triangles (seeded);
 * periodic = 1 pairs opposite sides (one physical group, SDG_BC_PERIODIC), else four groups
 * (bottom, right, top, left) with boundary_condition[0..3]. */
int sdg_mesh_generate_2d(double x0, double y0, double lx, double ly, int32_t nx, int32_t ny,
                         double jitter, double split_fraction, uint64_t seed, int32_t periodic,
                         const int32_t* boundary_condition, sdg_generated_mesh* out);
/* Annulus inner_radius <= r <= outer_radius of nr x ntheta curved elements with geometry order q (1..5):
 * element (i, j) spans [r_i, r_i+1] x [theta_j, theta_j+1]; its order-q Lagrange nodes lie on the exact
 * circles and rays (the curved meshes of the reference's cylinder drivers, examples/cylinder_2d_ceuler.cpp,
 * after setOrder(P)).  split_fraction of the quadrangles (seeded) are split into two curved triangles.  Two
 * boundary groups: the inner circle (1) and the outer circle (2), with boundary_condition[0..1]. */
int sdg_mesh_generate_annulus(double inner_radius, double outer_radius, int32_t nr, int32_t ntheta,
                              int32_t geometry_order, double split_fraction, uint64_t seed,
                              const int32_t* boundary_condition, sdg_generated_mesh* out);
/* 1D segment [x0, x0+lx], nx lines (examples/sod_1d_ceuler.cpp:68-82 and periodic_1d_ceuler.cpp:63-77:
 * gmsh transfinite curves); periodic = 1 joins the two end points (one group, SDG_BC_PERIODIC), else two
 * groups (x0 end, x0+lx end) with boundary_condition[0..1]. */
int sdg_mesh_generate_1d(double x0, double lx, int32_t nx, int32_t periodic, const int32_t* boundary_condition,
                         sdg_generated_mesh* out);
/* 3D box, nx x ny x nz hexahedra; periodic = 1 pairs opposite faces, else six groups
 * (x-, x+, y-, y+, z-, z+). */
int sdg_mesh_generate_3d(double x0, double y0, double z0, double lx, double ly, double lz, int32_t nx,
                         int32_t ny, int32_t nz, int32_t periodic, const int32_t* boundary_condition,
                         sdg_generated_mesh* out);
/* The same box with every hexahedron split into six tetrahedra around its lowest-to-highest diagonal
 * (conforming, periodic-compatible); boundary elements are triangles in the same six groups. */
int sdg_mesh_generate_3d_tetrahedra(double x0, double y0, double z0, double lx, double ly, double lz,
                                    int32_t nx, int32_t ny, int32_t nz, int32_t periodic,
                                    const int32_t* boundary_condition, sdg_generated_mesh* out);
/* Read a gmsh MSH 4.1 ASCII file (first-order or high-order elements).  A 2D mesh, or a 3D mesh of
 * hexahedra, of order q > 1 keeps every element's nodes as its curved geometry (geometry_order q); 1D meshes
 * and tetrahedra are read by their primary vertices (straight-sided).  Physical groups of dimension d-1 (points in 1D) become boundary groups
 * in file order. */
int sdg_mesh_read_msh(const char* path, sdg_generated_mesh* out);
int sdg_mesh_free(sdg_generated_mesh* mesh);

/* Artificial viscosity of the current state at every mesh node (the reference's node_artificial_viscosity_,
 * SpatialDiscrete.cpp:37-192): the sensor, the max over each node's elements.  Zeros without shock capturing.
 * out: [node_count]. */
int sdg_get_node_artificial_viscosity(sdg_handle* handle, double* out);

/* ---- raw-binary solution files (the reference's writeRawBinary / LastStep and SpecificFile restarts,
 * src/View/RawBinary.cpp:42-191, src/Solver/InitialCondition.cpp:40-80) ---------------------------------
 * u64 ZSTD_compressBound(payload) + one zstd level-1 frame; payload per element the column-major
 * (d+2) x Nb modal coefficients (Navier-Stokes: then the (d+2)*d x Nb gradient coefficients of the last
 * stage input), then per boundary face its parent's coefficients and gradient (BR1: the element's; BR2: its
 * volume gradient plus the lift of that face, RawBinary.cpp:98-112), in the order of
 * sdg_set_boundary_face_order, then one artificial viscosity value per mesh node (zero without shock
 * capturing).  BR2 records of parents with wall faces need the last gradient pass's input state:
 * SDG_ERR_UNSUPPORTED under forward Euler, which updates in place, and after an adjoint call until the next
 * step.  Needs libzstd.so.1 at run time (else SDG_ERR_UNSUPPORTED).
 * lower_order = 1 reads a file written at order P-1 into the leading coefficients (SpecificFile). */
int sdg_write_raw_binary(sdg_handle* handle, const char* path);
/* The caller's boundary-face order for the boundary block of raw-binary files: faces[k] = (element type,
 * element index within its type, local face) of the caller's k-th boundary face, every boundary face once.
 * The reference writes that block in its own adjacency order (the boundary entries of
 * AdjacencyElementMesh::element_, src/Mesh/Adjacency.cpp:466-485, written by src/View/RawBinary.cpp:120-154);
 * a shim passes that order here (parent_index_each_type_, adjacency_sequence_in_parent_ and the parent's type
 * of each boundary adjacency element) so that the reference's View reads the file unchanged.  Without it the
 * block follows this library's boundary-face order. */
int sdg_set_boundary_face_order(sdg_handle* handle, int64_t count, const int32_t* faces);
int sdg_read_raw_binary(sdg_handle* handle, const char* path, int32_t lower_order);

/* ---- launch shapes: CUDA-graph replay and the autotuner -------------------------------------------
 * sdg_step replays a CUDA graph of one full step (all stages and the relative-error reduction),
 * captured on first use and again when dt or a tile shape changes; enable = 0 issues the launches
 * one by one instead (kernel timing always does).  The reference has no equivalent: its step is a
 * oneTBB loop (src/Solver/TimeIntegration.cpp:326-350). */
int sdg_set_graph(sdg_handle* handle, int32_t enable);
/* Check of the failure detection of the device waits.  The tensor-block stage kernels stage each element
 * tile with TMA bulk copies that complete on an mbarrier, and wait for it at most `wait_limit` try_wait
 * rounds (0: the default, 2^24).  extra_expected_bytes > 0 (at most 65536) makes them declare that many
 * bytes beyond what their copies carry, so the wait can end only by its limit: every copy still lands, the
 * kernel withdraws the extra bytes, waits (bounded) until its copies have landed, flags the timeout and
 * returns, and the call reports SDG_ERR_TIMEOUT.  Nothing faults and no wait is unbounded.  The timeout
 * is sticky: the handle's state is no longer a valid step result; create a new handle.  (0, 0) restores the
 * normal kernels.  The reference has no equivalent (its only detection is the NaN check,
 * src/Utils/SystemControl.cpp:185-191). */
int sdg_set_wait_check(sdg_handle* handle, uint32_t wait_limit, uint32_t extra_expected_bytes);
/* Elements per CTA and threads per CTA of block `block`'s stage kernel and gradient kernel. */
int sdg_get_tile(const sdg_handle* handle, int32_t block, int32_t* elements_per_cta, int32_t* threads,
                 int32_t* gradient_elements_per_cta, int32_t* gradient_threads);
int sdg_set_tile(sdg_handle* handle, int32_t block, int32_t elements_per_cta, int32_t threads,
                 int32_t gradient_elements_per_cta, int32_t gradient_threads);
/* Autotuner: times every admissible tile of each block's stage kernel (and, for Navier-Stokes, its
 * gradient kernel) on the handle's current state and keeps the fastest.  Results are cached per
 * (device, kernel variant) for the process; flags bit 0 re-times cached variants.  The state is not
 * changed.  Tiles change only how elements are grouped into CTAs: the state a step produces is the
 * same bit for bit; the relative-error sums are regrouped (round-off only). */
#define SDG_AUTOTUNE_RETIME 1
int sdg_autotune(sdg_handle* handle, int32_t flags);

/* ---- batched solves: many independent problems in one set of launches -----------------------------
 * A batch advances `count` handles (any mix of meshes, element types, orders, Euler / Navier-Stokes,
 * physical constants; all on one device) together.  Per RK stage, every kernel class of every
 * (element type, order, affine, viscous) variant runs as ONE persistent launch over a work list of
 * (instance argument set, tile) items spanning all instances; independent launches of one dependency
 * level run on forked streams, and the full step is captured in a CUDA graph.  The handles stay
 * usable on their own; the batch does not own them.  Each instance's results (state, relative error,
 * status) are exactly those of sdg_step on the handle with the same tiles. */
typedef struct sdg_batch sdg_batch;
typedef struct sdg_batch_counts {
  int32_t instance_count;
  int32_t launches_per_step;          /* batched kernel launches per step (graph nodes)             */
  int32_t sequential_launches_per_step; /* launches per step when each instance runs alone         */
  int32_t persistent_ctas_per_sm;     /* CTAs per SM of the persistent launches (0: one per item)   */
  int64_t work_items_per_step;
  int64_t element_count;
  int64_t degree_of_freedom_count;
  int32_t stage_count;                /* RK stages per step of the instance with the most           */
} sdg_batch_counts;
/* Instances may be host-only handles (device < 0): the batch then only plans (sdg_batch_get_counts). */
int sdg_batch_create(sdg_handle* const* instances, int32_t count, sdg_batch** batch);
int sdg_batch_destroy(sdg_batch* batch);
int sdg_batch_get_counts(const sdg_batch* batch, sdg_batch_counts* counts);
/* dt of every instance, [count]; required before the first step, cheap to change (no re-capture). */
int sdg_batch_set_delta_time(sdg_batch* batch, const double* delta_time);
/* persistent CTAs per SM (0 = one CTA per work item); the autotuner picks it. */
int sdg_batch_set_persistence(sdg_batch* batch, int32_t ctas_per_sm);
/* step_count steps of every instance: graph replay of the batched launches (enqueued on the batch's
 * stream; sdg_batch_synchronize waits and checks every instance's status). */
int sdg_batch_step_async(sdg_batch* batch, int32_t step_count);
/* The same steps as one-instance launches, instance after instance on the batch's stream (the
 * comparison baseline: what the instances cost without batching). */
int sdg_batch_step_sequential_async(sdg_batch* batch, int32_t step_count);
int sdg_batch_synchronize(sdg_batch* batch);
/* Autotuner over the batch: each distinct variant's tiles (sdg_autotune on the first instance that
 * has it, shared by the rest), then the persistence; instance states are restored afterwards. */
int sdg_batch_autotune(sdg_batch* batch, int32_t flags);
int sdg_batch_get_stream(const sdg_batch* batch, void** stream);
const char* sdg_batch_last_error(const sdg_batch* batch);

/* ---- derivatives: tangent-linear model and discrete adjoint ---------------------------------------
 * Exact derivatives of the discrete scheme the forward path runs (the reference has none): for the
 * residual R(U) = du/dt and for whole SSP-RK trajectories, with respect to the state and to the dynamic
 * viscosity mu.  All vectors are in the volume-point layout of sdg_set_state_point ([point][d+2],
 * conserved variables; cotangents are mapped by the transposes of its point <-> state conversions, so the VJP
 * is the transpose of the JVP in that layout).  Supported: compressible or incompressible Euler and
 * Navier-Stokes (BR1, BR2) on every element block (lines, triangles -- straight or curved --, quadrangles --
 * parallelogram, bilinear or curved --, tetrahedra (P1-P3), hexahedra -- parallelepiped, trilinear or curved
 * --, hybrid meshes), the Boussinesq source, any boundary faces; with artificial viscosity
 * SDG_ERR_UNSUPPORTED. */
/* w_q |J|_q of every volume point: integral of f = sum over points of weight * f (functionals). */
int sdg_volume_point_weight(sdg_handle* handle, double* weight);
/* Change the dynamic viscosity (and kappa = cp mu / Pr) of a Navier-Stokes handle. */
int sdg_set_viscosity(sdg_handle* handle, double dynamic_viscosity);
/* rate_tangent = R'(U) tangent + dR/dmu viscosity_tangent at the current state U. */
int sdg_jvp_residual(sdg_handle* handle, const double* tangent, double viscosity_tangent, double* rate_tangent);
/* cotangent = R'(U)^T rate_cotangent, viscosity_cotangent = <rate_cotangent, dR/dmu> (may be NULL). */
int sdg_vjp_residual(sdg_handle* handle, const double* rate_cotangent, double* cotangent,
                     double* viscosity_cotangent);
/* Advance step_count steps of size delta_time (as sdg_step) and carry the tangent of the state along:
 * tangent_out = dU_N/dU_0 tangent_in + dU_N/dmu viscosity_tangent. */
int sdg_jvp_steps(sdg_handle* handle, int32_t step_count, double delta_time, const double* tangent_in,
                  double viscosity_tangent, double* tangent_out);
/* Discrete adjoint of step_count steps from the current state U_0 (the state is U_N on return, as after
 * sdg_step): initial_cotangent = (dU_N/dU_0)^T final_cotangent, viscosity_cotangent =
 * (dU_N/dmu)^T final_cotangent.  The state is kept every checkpoint_interval steps on the forward sweep
 * and each interval's stage states are recomputed from its checkpoint on the way back. */
int sdg_adjoint_steps(sdg_handle* handle, int32_t step_count, double delta_time, int32_t checkpoint_interval,
                      const double* final_cotangent, double* initial_cotangent, double* viscosity_cotangent);
/* The same trajectory in two calls, for callers that need U_N before choosing the cotangent (a loss
 * evaluated on U_N, an autograd engine): sdg_forward_steps advances step_count steps keeping the
 * checkpoints, sdg_adjoint_recorded then runs only the reverse sweep of that trajectory (the state must
 * not have changed in between: SDG_ERR_STATE). */
int sdg_forward_steps(sdg_handle* handle, int32_t step_count, double delta_time, int32_t checkpoint_interval);
int sdg_adjoint_recorded(sdg_handle* handle, const double* final_cotangent, double* initial_cotangent,
                         double* viscosity_cotangent);
/* Cotangent of the ghost primitive (rho, u, T) of every boundary point ([boundary_point_count][d+2], the order
 * of sdg_boundary_point_coordinate) accumulated by the last sdg_vjp_residual / sdg_adjoint_steps /
 * sdg_adjoint_recorded (and the ghost part left by sdg_surface_force_cotangent for Navier-Stokes walls): the
 * gradient with respect to the boundary (freestream) states. */
int sdg_adjoint_boundary_cotangent(sdg_handle* handle, double* cotangent);
/* Surface force of boundary group `physical` (1-based mesh physical index) on the current state: the sum over its
 * face points of w |J_f| (p n - tau n) from the interior traces, n out of the fluid (the reference's View force,
 * VariableConvertor.cpp:883-906).  force: [dimension]. */
int sdg_surface_force(sdg_handle* handle, int32_t physical, double* force);
/* Cotangent of direction . force with respect to the state ([volume_points][nv], the layout of the
 * adjoint's final cotangent): pressure and (Navier-Stokes) viscous stress through the gradient traces. */
int sdg_surface_force_cotangent(sdg_handle* handle, int32_t physical, const double* direction, double* cotangent);
/* Trajectory store (enable = 1; default 0): the forward sweep of sdg_adjoint_steps / sdg_forward_steps keeps
 * every stage input of every step in device memory when it fits (step_count x stages states, with 2 GiB left
 * free), and the reverse sweep reads them instead of recomputing each checkpoint interval from its checkpoint:
 * it then re-forms only the traces and (Navier-Stokes) the gradient pass of each stage input.  Without room the
 * checkpoint scheme runs.  Results are bit-identical between the two schemes. */
int sdg_set_adjoint_trajectory_store(sdg_handle* handle, int32_t enable);
/* Device bytes held for checkpoints, stage states and (Navier-Stokes, when HBM has room) the forward quantities
 * of one segment's stage inputs (grown on demand, released with the handle). */
int sdg_adjoint_memory(sdg_handle* handle, int64_t* bytes);

#ifdef __cplusplus
}
#endif

#endif /* SDG_GPU_H_ */
