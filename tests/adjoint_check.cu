// Host-side check of the reverse-mode far-pair derivatives (adjoint.cuh):
// the vertex gradient of S = Re sum C0 H0 + C1 H1 against central
// differences of the forward moments (pair_moments + vec_combine, the FP64
// far field's arithmetic), and the per-slot partial sums against direct sums.
// Prints the largest relative errors.
#include <cmath>
#include <cstdio>
#include "../scuff-em_gb300/csrc/adjoint.cuh"
using namespace gbem;

// the 6-point rule of the far field (libs/libTriInt/TCR.cc:83-91)
static const double RULE6[18] = {
    0.0915762135098, 0.0915762135098, 0.0549758718276, 0.8168475729805, 0.0915762135098, 0.0549758718276,
    0.0915762135098, 0.8168475729805, 0.0549758718276, 0.1081030181681, 0.4459484909160, 0.1116907948390,
    0.4459484909160, 0.1081030181681, 0.1116907948390, 0.4459484909160, 0.4459484909160, 0.1116907948390};

static double urand(unsigned* s) {
  *s = *s * 1664525u + 1013904223u;
  return (*s >> 8) * (1.0 / 16777216.0);
}

static void forward(const double* Va, const double* Vb, cx<double> k, const cx<double>* C0, const cx<double>* C1,
                    cx<double>* H0, cx<double>* H1) {
  PairGeom<double> g;
  for (int c = 0; c < 3; c++) {
    g.D0[c] = Va[c] - Vb[c];
    g.Aa[c] = Va[3 + c] - Va[c]; g.Ba[c] = Va[6 + c] - Va[c];
    g.Ab[c] = Vb[3 + c] - Vb[c]; g.Bb[c] = Vb[6 + c] - Vb[c];
  }
  cx<double> MG[9], MP[9];
  pair_moments<double, 0>(g, k, RULE6, 6, MG, MP);
  VecMoments<double> vm;
  vec_moments(g, MG, MP, &vm);
  const cx<double> m4 = cdiv(mk(-4.0, 0.0), k * k);
  for (int ja = 0; ja < 3; ja++)
    for (int jb = 0; jb < 3; jb++) vec_combine(g, vm, ja, jb, m4, &H0[3 * ja + jb], &H1[3 * ja + jb]);
}

static double energy(const double* Va, const double* Vb, cx<double> k, const cx<double>* C0, const cx<double>* C1) {
  cx<double> H0[9], H1[9];
  forward(Va, Vb, k, C0, C1, H0, H1);
  double e = 0.0;
  for (int m = 0; m < 9; m++) e += (C0[m] * H0[m] + C1[m] * H1[m]).re;
  return e;
}

int main() {
  unsigned seed = 777;
  double e_grad = 0.0, e_slot = 0.0;
  for (int t = 0; t < 40; t++) {
    double V[18];
    // panel a near the origin, panel b 4.5..9 radii away in a random direction
    for (int i = 0; i < 9; i++) V[i] = 0.3 * (urand(&seed) - 0.5);
    double dir[3] = {urand(&seed) - 0.5, urand(&seed) - 0.5, urand(&seed) - 0.5};
    const double dn = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const double dist = 1.0 + 1.5 * urand(&seed);
    for (int j = 0; j < 3; j++)
      for (int c = 0; c < 3; c++) V[9 + 3 * j + c] = dist * dir[c] / dn + 0.3 * (urand(&seed) - 0.5);
    const cx<double> k = mk(0.5 + 4.0 * urand(&seed), (t % 3 == 0) ? 0.0 : 0.3 * urand(&seed));
    cx<double> C0[9], C1[9];
    for (int m = 0; m < 9; m++) {
      C0[m] = mk(urand(&seed) - 0.5, urand(&seed) - 0.5);
      C1[m] = mk(urand(&seed) - 0.5, urand(&seed) - 0.5);
    }
    double gA[9] = {0}, gB[9] = {0}, Er[3], Ec[3];
    far_pair_vjp(V, V + 9, k, C0, C1, RULE6, 6, gA, gB, Er, Ec);
    double g[18], gmax = 0.0;
    for (int i = 0; i < 9; i++) { g[i] = gA[i]; g[9 + i] = gB[i]; }
    for (int i = 0; i < 18; i++) gmax = fmax(gmax, fabs(g[i]));
    for (int i = 0; i < 18; i++) {
      const double h = 1e-5;
      double Vp[18], Vm[18];
      for (int q = 0; q < 18; q++) Vp[q] = Vm[q] = V[q];
      Vp[i] += h; Vm[i] -= h;
      const double fd = (energy(Vp, Vp + 9, k, C0, C1) - energy(Vm, Vm + 9, k, C0, C1)) / (2 * h);
      e_grad = fmax(e_grad, fabs(fd - g[i]) / gmax);
    }
    cx<double> H0[9], H1[9];
    forward(V, V + 9, k, C0, C1, H0, H1);
    double smax = 0.0, er[3] = {0, 0, 0}, ec[3] = {0, 0, 0};
    for (int ja = 0; ja < 3; ja++)
      for (int jb = 0; jb < 3; jb++) {
        const double s = (C0[3 * ja + jb] * H0[3 * ja + jb] + C1[3 * ja + jb] * H1[3 * ja + jb]).re;
        er[ja] += s; ec[jb] += s;
      }
    for (int j = 0; j < 3; j++) smax = fmax(smax, fmax(fabs(er[j]), fabs(ec[j])));
    for (int j = 0; j < 3; j++) e_slot = fmax(e_slot, fmax(fabs(er[j] - Er[j]), fabs(ec[j] - Ec[j])) / smax);
  }
  printf("grad %.3e\nslot %.3e\n", e_grad, e_slot);
  return 0;
}
