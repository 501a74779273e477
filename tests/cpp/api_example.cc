// Exercises include/muspectre_gb300.hh the way a C++ user of µSpectre's API would.
//   api_example cpu   no GPU needed: error mapping (ProjectionError on an even grid)
//   api_example gpu   the README example (51x51 small strain, hard disc), printing
//                     success, Newton and CG counts and the homogenised stress
#include <cmath>
#include <cstdio>
#include <string>

#include "muspectre_gb300.hh"

using namespace muSpectre::gpu;

int main(int argc, char **argv) {
  const std::string mode = argc > 1 ? argv[1] : "cpu";
  if (mode == "cpu") {
    try {
      auto cell = make_cell<2>({4, 4}, {1., 1.}, Formulation::finite_strain);
      std::puts("no ProjectionError for an even grid");
      return 1;
    } catch (const ProjectionError &e) {
      std::printf("ProjectionError: %s\n", e.what());
    }
    std::printf("version %d\n", musg_version());
    return 0;
  }
  auto rve = make_cell<2>({51, 51}, {7., 5.}, Formulation::small_strain);
  const Communicator &comm = rve->get_communicator();  // single rank, as without MPI
  if (comm.rank() != 0 || comm.size() != 1 || comm.sum(2.5) != 2.5) {
    std::puts("unexpected communicator");
    return 1;
  }
  auto &hard = MaterialLinearElastic1<2>::make(*rve, "hard", 10e9, .33);
  auto &soft = MaterialLinearElastic1<2>::make(*rve, "soft", 70e9, .33);
  for (size_t i = 0; i < rve->size(); ++i) {
    const auto c = rve->get_ccoord(i);
    const double dx = c[0] - 25, dy = c[1] - 25;
    if (std::sqrt(dx * dx + dy * dy) < 10) hard.add_pixel(c);
    else soft.add_pixel(c);
  }
  SolverCG cg(*rve, 1e-8, 401);
  const std::vector<Real> del0 = {0., 0., 0., 0.03};  // [[0, 0], [0, .03]], column-major
  const OptimizeResult r = newton_cg(*rve, del0, cg, 1e-5, 2.0);
  const std::vector<Real> s = rve->homogenised_stress();
  std::printf("%d %u %u %.17g %.17g %.17g %.17g\n", int(r.success), r.nb_it, r.nb_fev, s[0], s[1], s[2], s[3]);
  SolverCG one(*rve, 1e-12, 1);
  try {
    newton_cg(*rve, del0, one, 1e-5, 2.0);
    std::puts("no ConvergenceError");
    return 1;
  } catch (const ConvergenceError &) {
    std::puts("ConvergenceError");
  }
  return 0;
}
