/*
 * Oracle (test infrastructure only): restatement of the svFSILS NS block
 * solver (L/NSSOLVER.f, L/GE.f, L/CGRAD.f:51-123, L/GMRES.f:51-169).
 */
#include "orc.h"

#include <stdio.h>
#include <stdlib.h>

void orc_nssolver(orc_lhs *lhs, orc_ls *ls, int dof, const double *Val, double *Ri) {
  (void)lhs; (void)ls; (void)dof; (void)Val; (void)Ri;
  fprintf(stderr, "oracle: NS solver not restated yet\n");
  abort();
}
