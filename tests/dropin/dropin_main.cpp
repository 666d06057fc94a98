// dropin_main.cpp -- a caller of the reference's own MDSystem class
// (src/library/MDSystem.h of vlvovch/lennard-jones-cuda), written the way
// its GUI and task programs use it: configure with useCUDA on, construct,
// integrate, read the observables.  tests/test_dropin_link.py compiles it
// with the reference's unmodified MDSystem.cpp and splinefunction.cpp under
// -DUSE_CUDA_TOOLKIT and links the result against liblj_gb300.so, which then
// provides every CUDA entry point MDSystem.cpp declares
// (MDSystem.cpp:9-25) in place of the reference's MDSystem.cu.
#include <cstdio>

#include "MDSystem.h"

int main() {
  MDSystem::MDSystemConfiguration config;
  config.N = 256;
  config.T0 = 1.0;
  config.rho = 0.5;
  config.useCUDA = true;
  MDSystem syst(config);
  for (int i = 0; i < 10; ++i) syst.Integrate(0.005);
  std::printf("U=%.10g T=%.10g P=%.10g\n", syst.U, syst.T, syst.P);
  return 0;
}
