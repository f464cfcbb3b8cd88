// C++23 host mirror of SubrosaDG's Solver<SimulationControl> / System<SimulationControl> over the C ABI of
// include/sdg_gpu.h.  Header-only; link with libsdg_gpu.so.
//
// GpuSolver<Control> has the members System<SC>::solve drives on the reference's Solver<SC>
// (src/Solver/SolveControl.cpp:327-436): initializeSolver, calculateDeltaTime, stepSolver, writeRawBinary and
// relative_error_.  System<Control> mirrors the reference facade (src/Utils/SystemControl.cpp:42-236: setMesh,
// addBoundaryCondition, setThermodynamicModel, setTransportModel, setTimeIntegration, setDeltaTime,
// setViewConfig, synchronize, solve) with the solve loop's outputs (error.txt lines, raw-binary files every
// io_interval steps, the NaN stop, SystemControl.cpp:159-195).  Mesh, PhysicalModel and TimeIntegration are
// plain stand-ins for the reference objects that carry the same data: a driver that builds them (from gmsh in
// the reference, from the library's generators or MSH reader here) steps on the GPU with no other change.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <filesystem>
#include <format>
#include <fstream>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sdg_gpu.h"

namespace sdg_cpp {

// Compile-time configuration, the runtime-free part of the reference's SimulationControl
// (src/Solver/SimulationControl.cpp:1197-1279); values are the reference's enum values (src/Utils/Enum.cpp).
// BoundaryTime: 0 steady, 1 time-varying ghost states (BoundaryTimeEnum, src/Utils/Enum.cpp:102-105).
template <int Dimension, int PolynomialOrder, int Equation, int ConvectiveFlux, int ViscousFlux = SDG_VISCOUS_NONE,
          int TimeIntegration = SDG_SSPRK3, int BoundaryTime = 0>
struct Control {
  static constexpr int kBoundaryTime = BoundaryTime;
  static constexpr int kDimension = Dimension;
  static constexpr int kPolynomialOrder = PolynomialOrder;
  static constexpr int kEquationModel = Equation;
  static constexpr int kConvectiveFlux = ConvectiveFlux;
  static constexpr int kViscousFlux = ViscousFlux;
  static constexpr int kTimeIntegration = TimeIntegration;
  static constexpr int kConservedVariableNumber = Dimension + 2;
  static constexpr int kPrimitiveVariableNumber = Dimension + 2;
};

// First-order mesh arrays in gmsh vertex order (the stand-in of Mesh<SC> after readMeshElement,
// src/Mesh/ReadControl.cpp:293-335).
struct Mesh {
  int dimension = 2;
  std::vector<double> node;  // [n][3]
  std::vector<int32_t> line, triangle, quadrangle, tetrahedron, hexahedron;
  std::vector<int32_t> boundary_node, boundary_physical, physical_boundary_condition, periodic_master;
  // curved meshes (setOrder(P), ReadControl.cpp:243-256): geometry order q > 1 and each element's gmsh-ordered
  // order-q nodes
  int geometry_order = 1;
  std::vector<int32_t> triangle_geometry, quadrangle_geometry, hexahedron_geometry;

  sdg_mesh view() const {
    sdg_mesh m{};
    m.dimension = dimension;
    m.node_count = int64_t(node.size() / 3);
    m.node_coordinate = node.data();
    m.periodic_master = periodic_master.empty() ? nullptr : periodic_master.data();
    m.triangle_count = int64_t(triangle.size() / 3);
    m.triangle_node = triangle.data();
    m.quadrangle_count = int64_t(quadrangle.size() / 4);
    m.quadrangle_node = quadrangle.data();
    m.hexahedron_count = int64_t(hexahedron.size() / 8);
    m.hexahedron_node = hexahedron.data();
    m.boundary_count = int64_t(boundary_physical.size());
    m.boundary_node = boundary_node.data();
    m.boundary_physical = boundary_physical.data();
    m.physical_count = int32_t(physical_boundary_condition.size());
    m.physical_boundary_condition = physical_boundary_condition.data();
    m.line_count = int64_t(line.size() / 2);
    m.line_node = line.data();
    m.tetrahedron_count = int64_t(tetrahedron.size() / 4);
    m.tetrahedron_node = tetrahedron.data();
    if (geometry_order > 1) {
      m.geometry_order = geometry_order;
      m.triangle_geometry_node = triangle_geometry.empty() ? nullptr : triangle_geometry.data();
      m.quadrangle_geometry_node = quadrangle_geometry.empty() ? nullptr : quadrangle_geometry.data();
      m.hexahedron_geometry_node = hexahedron_geometry.empty() ? nullptr : hexahedron_geometry.data();
    }
    return m;
  }

  // Copies a mesh the library generated or read (sdg_mesh_generate_*, sdg_mesh_read_msh) and frees it.
  static Mesh fromGenerated(sdg_generated_mesh& g) {
    const sdg_mesh& m = g.mesh;
    Mesh out;
    out.dimension = m.dimension;
    const auto take = [](auto* p, int64_t n, auto& v) { if (p && n > 0) v.assign(p, p + n); };
    const int nbv = m.dimension == 1 ? 1 : (m.dimension == 2 ? 2 : 4);
    take(m.node_coordinate, m.node_count * 3, out.node);
    take(m.periodic_master, m.node_count, out.periodic_master);
    take(m.line_node, m.line_count * 2, out.line);
    take(m.triangle_node, m.triangle_count * 3, out.triangle);
    take(m.quadrangle_node, m.quadrangle_count * 4, out.quadrangle);
    take(m.tetrahedron_node, m.tetrahedron_count * 4, out.tetrahedron);
    take(m.hexahedron_node, m.hexahedron_count * 8, out.hexahedron);
    take(m.boundary_node, m.boundary_count * nbv, out.boundary_node);
    take(m.boundary_physical, m.boundary_count, out.boundary_physical);
    take(m.physical_boundary_condition, int64_t(m.physical_count), out.physical_boundary_condition);
    if (m.geometry_order > 1) {
      const int64_t q = m.geometry_order;
      out.geometry_order = int(q);
      take(m.triangle_geometry_node, m.triangle_count * (q + 1) * (q + 2) / 2, out.triangle_geometry);
      take(m.quadrangle_geometry_node, m.quadrangle_count * (q + 1) * (q + 1), out.quadrangle_geometry);
      take(m.hexahedron_geometry_node, m.hexahedron_count * (q + 1) * (q + 1) * (q + 1), out.hexahedron_geometry);
    }
    sdg_mesh_free(&g);
    return out;
  }
};

// Thermodynamic / transport constants (PhysicalModel<SC>, src/Solver/PhysicalModel.cpp:40-165).
struct PhysicalModel {
  double specific_heat_ratio = 1.4;  // the reference's constexpr (PhysicalModel.cpp:45)
  double specific_heat_constant_pressure = 0.0, specific_heat_constant_volume = 0.0;
  double dynamic_viscosity = 0.0, prandtl_number = 0.71;
  int transport_model = SDG_TRANSPORT_CONSTANT;
};

// TimeIntegration<SC> (src/Solver/TimeIntegration.cpp:30-43): CFL number, step range, dt.
struct TimeIntegration {
  double courant_friedrichs_lewy_number = 1.0;
  int iteration_start = 0, iteration_end = 0;
  double delta_time = 0.0;
  bool fixed_delta_time = false;  // System::setDeltaTime
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc, const sdg_handle* h, const char* call) {
  if (rc != SDG_OK) throw Error(rc, std::format("{}: {}", call, sdg_last_error(h)));
}

// The GPU Solver<SC>: one sdg_handle on one device (device < 0: host-only handle, no GPU touched).
template <class SC>
class GpuSolver {
 public:
  using Point = std::array<double, 3>;
  using Primitive = std::array<double, SC::kPrimitiveVariableNumber>;
  std::array<double, SC::kConservedVariableNumber> relative_error_{};

  GpuSolver() = default;
  GpuSolver(const GpuSolver&) = delete;
  GpuSolver& operator=(const GpuSolver&) = delete;
  ~GpuSolver() {
    if (handle_) sdg_destroy(handle_);
  }

  // The driver's boundary state: boundary(x, time, physical index) (time 0 and unused for steady states).
  using BoundaryFunction = std::function<Primitive(const Point&, double, int)>;

  // Solver::initializeSolver (src/Solver/InitialCondition.cpp:85-149): build the problem, then the initial
  // state from the driver's primitive function at the volume points and the ghost states at the boundary
  // points at time 0.
  void initializeSolver(const Mesh& mesh, const PhysicalModel& pm, const std::function<Primitive(const Point&)>& ic,
                        const BoundaryFunction& boundary = {}, int device = 0) {
    const sdg_mesh m = mesh.view();
    sdg_config c{};
    c.polynomial_order = SC::kPolynomialOrder;
    c.equation = SC::kEquationModel;
    c.convective_flux = SC::kConvectiveFlux;
    c.viscous_flux = SC::kViscousFlux;
    c.time_integration = SC::kTimeIntegration;
    c.transport_model = pm.transport_model;
    c.specific_heat_ratio = pm.specific_heat_ratio;
    c.specific_heat_constant_pressure = pm.specific_heat_constant_pressure;
    c.specific_heat_constant_volume = pm.specific_heat_constant_volume;
    c.dynamic_viscosity = pm.dynamic_viscosity;
    c.prandtl_number = pm.prandtl_number;
    c.artificial_viscosity_factor = 1.0;
    check(sdg_create(&m, &c, device, &handle_), nullptr, "sdg_create");
    check(sdg_get_counts(handle_, &counts_), handle_, "sdg_get_counts");
    if (device < 0) return;  // host-only: adjacency, geometry and counts only
    const int nv = SC::kConservedVariableNumber;
    std::vector<double> x(size_t(counts_.volume_point_count) * 3), prim(size_t(counts_.volume_point_count) * nv);
    check(sdg_volume_point_coordinate(handle_, x.data()), handle_, "sdg_volume_point_coordinate");
    for (int64_t q = 0; q < counts_.volume_point_count; ++q) {
      const Primitive p = ic({x[q * 3], x[q * 3 + 1], x[q * 3 + 2]});
      for (int v = 0; v < nv; ++v) prim[size_t(q) * nv + v] = p[v];
    }
    check(sdg_set_initial_primitive(handle_, prim.data()), handle_, "sdg_set_initial_primitive");
    boundary_ = boundary;
    if (counts_.boundary_face_count > 0 && boundary_) {
      bx_.resize(size_t(counts_.boundary_point_count) * 3);
      bphys_.resize(size_t(counts_.boundary_face_count));
      check(sdg_boundary_point_coordinate(handle_, bx_.data(), bphys_.data()), handle_, "sdg_boundary_point_coordinate");
      updateBoundaryVariable(0.0);
    }
  }

  // Solver::updateBoundaryVariable (src/Solver/BoundaryCondition.cpp:29-74): ghost states of the boundary
  // points at `time`.
  void updateBoundaryVariable(double time) {
    if (bx_.empty()) return;
    const int nv = SC::kConservedVariableNumber;
    const int64_t nb = counts_.boundary_point_count;
    std::vector<double> bp(size_t(nb) * nv);
    for (int64_t q = 0; q < nb; ++q) {
      const Primitive p = boundary_({bx_[q * 3], bx_[q * 3 + 1], bx_[q * 3 + 2]}, time,
                                    bphys_[q / counts_.face_point_count]);
      for (int v = 0; v < nv; ++v) bp[size_t(q) * nv + v] = p[v];
    }
    check(sdg_set_boundary_primitive(handle_, bp.data()), handle_, "sdg_set_boundary_primitive");
  }

  // Solver::calculateDeltaTime (TimeIntegration.cpp:104-131).
  void calculateDeltaTime(TimeIntegration& ti) {
    check(sdg_calculate_delta_time(handle_, ti.courant_friedrichs_lewy_number, &ti.delta_time), handle_,
          "sdg_calculate_delta_time");
  }

  // Solver::stepSolver (TimeIntegration.cpp:326-350), then relative_error_ of the step (:279-324).
  void stepSolver(const TimeIntegration& ti) {
    check(sdg_step(handle_, 1, ti.delta_time), handle_, "sdg_step");
    check(sdg_relative_error(handle_, relative_error_.data()), handle_, "sdg_relative_error");
  }

  // Solver::writeRawBinary (src/View/RawBinary.cpp:156-191).
  void writeRawBinary(const std::filesystem::path& path) {
    check(sdg_write_raw_binary(handle_, path.c_str()), handle_, "sdg_write_raw_binary");
  }
  // InitialConditionEnum::LastStep / SpecificFile (InitialCondition.cpp:40-80).
  void readRawBinary(const std::filesystem::path& path, bool lower_order) {
    check(sdg_read_raw_binary(handle_, path.c_str(), lower_order ? 1 : 0), handle_, "sdg_read_raw_binary");
  }

  // Conserved state at the volume points, [volume_point_count][d+2].
  std::vector<double> statePoint() {
    std::vector<double> out(size_t(counts_.volume_point_count) * SC::kConservedVariableNumber);
    check(sdg_get_state_point(handle_, out.data()), handle_, "sdg_get_state_point");
    return out;
  }

  const sdg_counts& counts() const { return counts_; }
  sdg_handle* handle() const { return handle_; }

 private:
  sdg_handle* handle_ = nullptr;
  sdg_counts counts_{};
  BoundaryFunction boundary_;
  std::vector<double> bx_;       // boundary point coordinates
  std::vector<int32_t> bphys_;   // physical group of each boundary face
};

// The reference's System<SC> facade over GpuSolver<SC> (src/Utils/SystemControl.cpp:42-236).
template <class SC>
class System {
 public:
  using Primitive = typename GpuSolver<SC>::Primitive;
  using Point = typename GpuSolver<SC>::Point;

  void setMesh(Mesh mesh) { mesh_ = std::move(mesh); }
  // System::addBoundaryCondition<BC>(physical index) (SystemControl.cpp:76-80)
  void addBoundaryCondition(int condition, int physical_index) {
    auto& bc = mesh_.physical_boundary_condition;
    if (physical_index < 1 || physical_index > int(bc.size())) throw Error(SDG_ERR_INVALID_ARGUMENT, "physical index");
    bc[physical_index - 1] = condition;
  }
  void setThermodynamicModel(double cp, double cv) {  // SystemControl.cpp:82-88
    physical_model_.specific_heat_constant_pressure = cp;
    physical_model_.specific_heat_constant_volume = cv;
  }
  void setTransportModel(double mu) { physical_model_.dynamic_viscosity = mu; }  // SystemControl.cpp:98-103
  void setTimeIntegration(double cfl, std::array<int, 2> range = {0, 0}) {     // SystemControl.cpp:110-120
    time_integration_.courant_friedrichs_lewy_number = cfl;
    time_integration_.iteration_start = range[0];
    time_integration_.iteration_end = range[1];
  }
  void setDeltaTime(double dt) {  // SystemControl.cpp:122
    time_integration_.delta_time = dt;
    time_integration_.fixed_delta_time = true;
  }
  void setViewConfig(std::filesystem::path directory, std::string prefix, int io_interval = 0) {
    output_directory_ = std::move(directory);
    prefix_ = std::move(prefix);
    io_interval_ = io_interval;
  }
  void setInitialCondition(std::function<Primitive(const Point&)> f) { ic_ = std::move(f); }
  void setBoundaryCondition(typename GpuSolver<SC>::BoundaryFunction f) { bc_ = std::move(f); }

  // System::synchronize (SystemControl.cpp:146-157): problem setup and the initial state on `device`.
  void synchronize(int device = 0) { solver_.initializeSolver(mesh_, physical_model_, ic_, bc_, device); }

  // System::solve (SystemControl.cpp:159-195): dt (unless fixed), the step-0 raw-binary file, then steps
  // iteration_start+1 .. iteration_end with one error.txt line each (View/CommandLine.cpp:70-106: a header,
  // the zero line, then |{:^13.5e}| fields of time and relative errors), raw-binary files every io_interval
  // steps, and the stop when every relative error is NaN.  Returns the number of steps taken.
  int solve() {
    if (!time_integration_.fixed_delta_time) solver_.calculateDeltaTime(time_integration_);
    const double dt = time_integration_.delta_time;
    std::ofstream error;
    const int io = io_interval_ > 0 ? io_interval_ : time_integration_.iteration_end;
    if (!output_directory_.empty()) {
      std::filesystem::create_directories(output_directory_ / "raw");
      error.open(output_directory_ / "error.txt");
      solver_.writeRawBinary(rawPath(0));
      error << variableList() << '\n' << line(0.0, {}) << '\n';
    }
    int step = time_integration_.iteration_start;
    int iteration = 0;  // TimeIntegration::iteration_ (TimeIntegration.cpp:37): 0 until a step has been taken
    for (int i = time_integration_.iteration_start + 1; i <= time_integration_.iteration_end; ++i) {
      // BoundaryTimeEnum::TimeVarying: ghost states at the start of each step (TimeIntegration.cpp:333-335)
      if constexpr (SC::kBoundaryTime == 1) solver_.updateBoundaryVariable(iteration * dt);
      solver_.stepSolver(time_integration_);
      step = iteration = i;
      if (error.is_open()) {
        if (i % io == 0) solver_.writeRawBinary(rawPath(i));
        error << line(i * dt, solver_.relative_error_) << '\n';
      }
      bool all_nan = true;
      for (double e : solver_.relative_error_) all_nan = all_nan && std::isnan(e);
      if (all_nan) break;
    }
    return step - time_integration_.iteration_start;
  }

  GpuSolver<SC>& solver() { return solver_; }
  TimeIntegration& timeIntegration() { return time_integration_; }

 private:
  std::filesystem::path rawPath(int step) const {
    return output_directory_ / "raw" / std::format("{}_{}.zst", prefix_, step);
  }
  static std::string variableList() {
    const bool inc = SC::kEquationModel == SDG_INCOMPRESSIBLE_EULER || SC::kEquationModel == SDG_INCOMPRESSIBLE_NS;
    std::string out = std::format("|{:^13}|{:^13}|", "Time", "rho");
    for (int k = 0; k < SC::kDimension; ++k) out += std::format("{:^13}|", std::string("rho*") + "uvw"[k]);
    return out + std::format("{:^13}|", inc ? "rho*e" : "rho*E");
  }
  static std::string line(double time, const std::array<double, SC::kConservedVariableNumber>& e) {
    std::string out = std::format("|{:^13.5e}|", time);
    for (double x : e) out += std::format("{:^13.5e}|", x);
    return out;
  }

  Mesh mesh_;
  PhysicalModel physical_model_;
  TimeIntegration time_integration_;
  GpuSolver<SC> solver_;
  std::function<Primitive(const Point&)> ic_;
  typename GpuSolver<SC>::BoundaryFunction bc_;
  std::filesystem::path output_directory_;
  std::string prefix_;
  int io_interval_ = 0;
};

}  // namespace sdg_cpp
