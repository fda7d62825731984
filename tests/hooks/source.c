/* A specialsource + getdt_special test hook for the CPU oracle
 * (vo_register_source_fn): a force along x_1 that grows with x_1 and with
 * time, the work it does, and a damping of m_2,
 *   f = 0.02*(0.5+0.1*x_1)*(1+qtC),
 *   m_1 += qdt*(rho*f),  e += qdt*(m_1*f),  m_2 -= qdt*(0.05*m_2),
 * with the time step limit dt_mine = 0.05/(0.001 + max |m_1|/rho).  The same
 * formulas, in the same operation order, as the device hook in source.cu.
 * `user` carries the index of e (1 + ndir).  Build with -ffp-contract=off. */
void src_host(void* user, double qdt, double qtC, const double* wCT, double qt,
              double* w, const int* lo, const int* hi, const long* st, long N,
              const double* const* x) {
  (void)qt;
  const long e = (long)user;
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        const long ix = i + st[1] * j + st[2] * k;
        const double f = 0.02 * (0.5 + 0.1 * x[0][ix]) * (1.0 + qtC);
        w[ix + N] = w[ix + N] + qdt * (wCT[ix] * f);
        w[ix + e * N] = w[ix + e * N] + qdt * (wCT[ix + N] * f);
        if (e >= 3) w[ix + 2 * N] = w[ix + 2 * N] - qdt * (0.05 * wCT[ix + 2 * N]);
      }
}

double dt_host(void* user, const double* w, const int* lo, const int* hi, const long* st,
               long N, const double* const* x) {
  (void)user; (void)x;
  double m = 0.0;
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        const long ix = i + st[1] * j + st[2] * k;
        double v = w[ix + N] / w[ix];
        v = v < 0.0 ? -v : v;
        if (v > m) m = v;
      }
  return 0.05 / (0.001 + m);
}
