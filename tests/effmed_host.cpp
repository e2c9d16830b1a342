// Reads mean lab-frame tensors (sym, is_real, then 12 doubles: 00, 11, 22,
// 01, 02, 12 as re, im) from stdin and prints the engine's effective medium of each
// (sym, epsv re/im x 3, psi, theta, phi) on one line.
#include <cstdio>

#include "dtmm_effmed.h"

int main() {
  int sym, is_real;
  double t[12], out[10];
  while (std::scanf("%d %d", &sym, &is_real) == 2) {
    for (int i = 0; i < 12; ++i)
      if (std::scanf("%lf", &t[i]) != 1) return 1;
    eff_medium(t, sym, is_real != 0, out);
    for (int i = 0; i < 10; ++i) std::printf("%.17g%c", out[i], i == 9 ? '\n' : ' ');
  }
  return 0;
}
