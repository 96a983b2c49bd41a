// Test driver: a reference-shaped C++ program (cf. parallel/repulsive-vicsek.cpp
// data_gathering, :52-105) written against include/spp_box.hpp.  Reads the
// initial state from argv[1] (n float32 x, then y, then theta), runs the
// repulsive-ABP workload in chunks of Multi_Step, writes the polarization
// series to stdout and the final frame (operator<<) to argv[2].
#include <cstdio>
#include <fstream>
#include <iostream>
#include <vector>

#include "spp_box.hpp"

int main(int argc, char** argv) {
  if (argc < 5) {
    std::cerr << "usage: abp_driver state.f32 out.bin n L" << std::endl;
    return 2;
  }
  const int n = std::atoi(argv[3]);
  const double L = std::atof(argv[4]);
  std::vector<float> x(n), y(n), th(n);
  std::ifstream in(argv[1], std::ios::binary);
  in.read(reinterpret_cast<char*>(x.data()), sizeof(float) * n);
  in.read(reinterpret_cast<char*>(y.data()), sizeof(float) * n);
  in.read(reinterpret_cast<char*>(th.data()), sizeof(float) * n);
  if (!in) {
    std::cerr << "short input" << std::endl;
    return 2;
  }
  SppParams p;
  spp::check(spp_params_init(&p, SPP_MODEL_ABP), "spp_params_init");
  p.n = n;
  p.L = L;
  p.seed = 1;
  p.integrator = SPP_INT_RK2;
  p.force_law = SPP_FORCE_HARMONIC;
  p.align_mode = SPP_ALIGN_MEAN;
  p.k_rep = 10.0;
  p.r_rep = 1.0;
  p.g = 1.0;
  p.r_align = 1.0;
  p.Dr = 0.1;
  p.v0 = 1.0;
  p.dt = 0.005;
  p.skin = 0.3;
  try {
    spp::Box box(p);
    box.Init(x, y, th);
    for (int chunk = 0; chunk < 4; ++chunk) {
      box.Multi_Step(25);
      box.Save_Polarization(std::cout);
    }
    std::ofstream out(argv[2], std::ios::binary);
    out << box;
  } catch (const spp::Error& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
