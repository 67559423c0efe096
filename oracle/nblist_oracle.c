/* placeholder: CPU cluster-pair builder, filled in with the GPU list build */
#include "mspms_oracle.h"
int orc_nblist_build(const double *x, const double *y, const double *z, int natom, double lx,
                     double ly, double lz, double rlist, int *out_ncl, int *cluster_atoms,
                     int cluster_cap, long long *out_npairs, int *pairs, int *shifts,
                     long long pair_cap) {
    (void)x; (void)y; (void)z; (void)natom; (void)lx; (void)ly; (void)lz; (void)rlist;
    (void)cluster_atoms; (void)cluster_cap; (void)pairs; (void)shifts; (void)pair_cap;
    *out_ncl = 0; *out_npairs = 0;
    return -1;
}
