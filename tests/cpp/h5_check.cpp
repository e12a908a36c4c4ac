// Exercises include/sfd_h5.hpp from C++ (no GPU):
//   h5_check write <path>          write a fixed state file with saveStateFile
//   h5_check read <path> <N>       loadStateFile, print Z and phi (%.17g)
//   h5_check traj <path>           read a T / Y / x0 / y0 / pot0 trajectory and
//                                  check that Y[0] == [x0 | y0 | pot0]
#include <cstdio>
#include <string>

#include "sfd_h5.hpp"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  const std::string mode = argv[1], path = argv[2];
  try {
    if (mode == "write") {
      const size_t n = 8;
      std::vector<std::complex<double>> Z(n);
      std::vector<double> phi(n);
      for (size_t j = 0; j < n; ++j) {
        Z[j] = {0.25 * j, 0.5 * j - 1.0};
        phi[j] = 0.1 * j;
      }
      return sfd::saveStateFile(path, Z, phi, n, 0.25, 1e-3, 0.0, 2.0, 0.05, true);
    }
    if (mode == "read") {
      const size_t n = std::stoul(argv[3]);
      std::vector<std::complex<double>> Z;
      std::vector<double> phi;
      sfd::loadStateFile(path, Z, phi, n, 1.0);
      for (size_t j = 0; j < n; ++j) std::printf("%.17g %.17g %.17g\n", Z[j].real(), Z[j].imag(), phi[j]);
      return 0;
    }
    if (mode == "traj") {
      std::map<std::string, sfd::h5::Dataset> ds;
      std::map<std::string, sfd::h5::Attr> at;
      sfd::h5::read(path, ds, at);
      const auto &x0 = ds.at("x0"), &y0 = ds.at("y0"), &p0 = ds.at("pot0"), &Y = ds.at("Y"), &T = ds.at("T");
      const size_t n = x0.data.size();
      if (Y.shape.size() != 2 || Y.shape[0] != T.data.size() || Y.shape[1] != 3 * n) return 3;
      for (size_t j = 0; j < n; ++j)
        if (Y.data[j] != x0.data[j] || Y.data[n + j] != y0.data[j] || Y.data[2 * n + j] != p0.data[j]) return 4;
      std::printf("ok %zu %zu\n", (size_t)T.data.size(), n);
      return 0;
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 2;
}
