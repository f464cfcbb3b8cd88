// The reference's example driver examples/periodic_2d_ceuler.cpp on the GPU path, written against the C++
// mirror of System<SC> (gpu_solver.hpp) over the C ABI: 2D compressible Euler, P3 quadrangles, HLLC, SSP-RK3,
// the density wave rho = 1 + 0.2 sin(pi (x + y)), u = (0.7, 0.3), p = 1 on the periodic [0, 2]^2 of 10 x 10
// transfinite quadrangles, cp = 2.5, cv = 25/14, dt = 1e-3.  The mesh comes from the library's structured
// generator in place of gmsh (generateMesh of the example).
//
//   periodic_2d_ceuler <steps> <output directory> [io_interval] [--host-only]
//
// Writes <output>/error.txt and <output>/raw/periodic_2d_ceuler_<i>.zst as the reference's solve loop does, and
// <output>/state.f64: the conserved state at the volume points after the last step ([points][4] doubles).
// --host-only creates a host-only handle (device < 0) and prints the problem's counts: no GPU is touched.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <numbers>
#include <string>

#include "gpu_solver.hpp"

using SimulationControl = sdg_cpp::Control<2, 3, SDG_COMPRESSIBLE_EULER, SDG_FLUX_HLLC, SDG_VISCOUS_NONE, SDG_SSPRK3>;

int main(int argc, char* argv[]) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: %s <steps> <output directory> [io_interval] [--host-only]\n", argv[0]);
    return 2;
  }
  const int steps = std::atoi(argv[1]);
  const std::filesystem::path out = argv[2];
  const int io_interval = argc > 3 && argv[3][0] != '-' ? std::atoi(argv[3]) : 0;
  const bool host_only = std::string(argv[argc - 1]) == "--host-only";
  try {
    sdg_generated_mesh g{};
    sdg_cpp::check(sdg_mesh_generate_2d(0.0, 0.0, 2.0, 2.0, 10, 10, 0.0, 0.0, 0, 1, nullptr, &g), nullptr,
                   "sdg_mesh_generate_2d");
    sdg_cpp::System<SimulationControl> system;
    system.setMesh(sdg_cpp::Mesh::fromGenerated(g));
    system.addBoundaryCondition(SDG_BC_PERIODIC, 1);
    system.setThermodynamicModel(2.5, 25.0 / 14.0);
    system.setTimeIntegration(1.0, {0, steps});
    system.setDeltaTime(1.0e-3);
    system.setViewConfig(out, "periodic_2d_ceuler", io_interval);
    system.setInitialCondition([](const sdg_cpp::System<SimulationControl>::Point& x) {
      const double s = std::sin(std::numbers::pi * (x[0] + x[1]));
      return sdg_cpp::System<SimulationControl>::Primitive{1.0 + 0.2 * s, 0.7, 0.3, 1.4 / (1.0 + 0.2 * s)};
    });
    system.synchronize(host_only ? -1 : 0);
    const sdg_counts& c = system.solver().counts();
    if (host_only) {
      std::printf("elements %lld interior_faces %lld boundary_faces %lld volume_points %lld dof %lld\n",
                  static_cast<long long>(c.element_count), static_cast<long long>(c.interior_face_count),
                  static_cast<long long>(c.boundary_face_count), static_cast<long long>(c.volume_point_count),
                  static_cast<long long>(c.degree_of_freedom_count));
      return 0;
    }
    const int done = system.solve();
    const std::vector<double> state = system.solver().statePoint();
    std::ofstream(out / "state.f64", std::ios::binary)
        .write(reinterpret_cast<const char*>(state.data()), std::streamsize(state.size() * sizeof(double)));
    std::printf("steps %d relative_error", done);
    for (double e : system.solver().relative_error_) std::printf(" %.17g", e);
    std::printf("\n");
  } catch (const sdg_cpp::Error& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
