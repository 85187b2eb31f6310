// Stand-in for the reference's missing Units.hpp: only the Gaussian pair of its headers'
// division and migration times is needed to compile MD.cuh's force laws on the host.
#pragma once
struct Gaussian {
  double mu = 0.0;
  double sigma = 0.0;
};
