/* A specialeta test hook for the CPU oracle (vo_register_eta): a
 * resistivity that grows with x and with the current,
 *   eta = 0.005*(1+x_1^2) + 0.001*J_3^2,  gradeta = (0.01*x_1, 0, 0),
 * the same formula, in the same operation order, as the device hook in
 * eta.cu.  Build with -ffp-contract=off. */
void eta_host(void* user, const double* w, const double* const* cur,
              double* eta, double* const* gradeta, const int* lo,
              const int* hi, const long* st, long N, const double* const* x,
              int idirmin, double t) {
  (void)user; (void)w; (void)N; (void)idirmin; (void)t;
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        const long ix = i + st[1] * j + st[2] * k;
        const double x1 = x[0][ix], j3 = cur[2][ix];
        eta[ix] = 0.005 * (1.0 + x1 * x1) + 0.001 * (j3 * j3);
        if (gradeta[0]) {
          gradeta[0][ix] = 0.01 * x1;
          if (gradeta[1]) gradeta[1][ix] = 0.0;
          if (gradeta[2]) gradeta[2][ix] = 0.0;
        }
      }
}
