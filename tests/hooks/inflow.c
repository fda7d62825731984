/* A specialbound test hook for the CPU oracle (vo_register_bound): a
 * time-dependent inflow mixed with the edge value,
 *   w(ghost) = 0.5*(w(edge) + (1+0.1*iw)*(1+0.1*qt)) + 0.01*x_idim(ghost),
 * the same formula, in the same operation order, as the device hook in
 * inflow.cu.  Build with -ffp-contract=off. */
void inflow_bound_host(void* user, double* w, const int* lo, const int* hi,
                       const long* st, long N, const double* x, int iw,
                       int iB, double qt) {
  (void)user;
  const int idim = iB / 2, upper = iB % 2;
  const int e = upper ? lo[idim] - 1 : hi[idim] + 1; /* edge mesh layer */
  double* a = w + (long)iw * N;
  for (int k = lo[2]; k <= hi[2]; k++)
    for (int j = lo[1]; j <= hi[1]; j++)
      for (int i = lo[0]; i <= hi[0]; i++) {
        int c[3] = {i, j, k};
        const long ix = c[0] + st[1] * c[1] + st[2] * c[2];
        c[idim] = e;
        const long ie = c[0] + st[1] * c[1] + st[2] * c[2];
        a[ix] = 0.5 * (a[ie] + (1.0 + 0.1 * iw) * (1.0 + 0.1 * qt)) +
                0.01 * x[ix];
      }
}
