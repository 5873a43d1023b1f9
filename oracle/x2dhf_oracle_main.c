/*
 * x2dhf CPU oracle command-line driver -- TEST INFRASTRUCTURE ONLY.
 * Runs a reference-format input file through the oracle's SCF loop and
 * prints the per-iteration lines in the reference's layout
 * (src/doSCF.F90:872-885 formats).
 */
#include <stdio.h>
#include <stdlib.h>
#include "x2dhf_oracle.h"

int main(int argc, char **argv) {
  if (argc < 2) { fprintf(stderr, "usage: %s input.data\n", argv[0]); return 2; }
  FILE *f = fopen(argv[1], "rb");
  if (!f) { perror(argv[1]); return 2; }
  fseek(f, 0, SEEK_END); long n = ftell(f); fseek(f, 0, SEEK_SET);
  char *buf = (char *)malloc(n + 1);
  if (fread(buf, 1, n, f) != (size_t)n) { fclose(f); return 2; }
  buf[n] = 0; fclose(f);
  char err[256];
  x2o_state *s = x2o_from_input(buf, err, sizeof err);
  free(buf);
  if (!s) { fprintf(stderr, "input error: %s\n", err); return 1; }
  x2o_setup(s);
  printf("   Grid: nu=%d mu=%d  omega orb=%.3f pot=%.3f\n", x2o_nni(s), x2o_nmu(s), x2o_omega_orb(s), x2o_omega_pot(s));
  x2o_run_scf(s, 1);
  x2o_free(s);
  return 0;
}
