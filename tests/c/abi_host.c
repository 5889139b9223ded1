/* A plain C caller of the PNAMP C ABI, as a Fortran bind(C) shim or a C++ harness would
 * bind it: the host-only entry points (no device is touched), linked against the built
 * library. Prints the Rho2B table sizes of the pf shell (Z = N = 4) and the error texts. */
#include <stdio.h>
#include <string.h>

#include "pnamp_gpu.h"

int main(void) {
    /* pf shell: 0f7/2, 1p3/2, 0f5/2, 1p1/2 (n from 1), protons (t = -1) then neutrons */
    static const int orb_n[4] = {1, 2, 1, 2}, orb_l[4] = {3, 1, 3, 1}, orb_tj[4] = {7, 3, 5, 1};
    int t[64], n[64], l[64], tj[64], tm[64], k = 0;
    for (int s = 0; s < 2; ++s)
        for (int o = 0; o < 4; ++o)
            for (int m = orb_tj[o]; m >= -orb_tj[o]; m -= 2) {
                t[k] = s ? 1 : -1;
                n[k] = orb_n[o];
                l[k] = orb_l[o];
                tj[k] = orb_tj[o];
                tm[k] = m;
                ++k;
            }
    pnamp_space sp;
    memset(&sp, 0, sizeof sp);
    sp.nlev = k;
    sp.nprot = 4;
    sp.nneut = 4;
    sp.t = t;
    sp.n = n;
    sp.l = l;
    sp.twoj = tj;
    sp.twom = tm;
    int sizes[5];
    int rc = pnamp_rho2b_layout(&sp, sizes);
    if (rc != PNAMP_OK) {
        fprintf(stderr, "pnamp_rho2b_layout: %s\n", pnamp_strerror(rc));
        return 1;
    }
    printf("nlev %d blocks %d states %d elements %d quads %d terms %d\n", k, sizes[0], sizes[1], sizes[2],
           sizes[3], sizes[4]);
    if (pnamp_rho2b_layout(NULL, sizes) != PNAMP_ERR_ARG) return 2;
    printf("version %s\n", pnamp_version());
    printf("err %s\n", pnamp_strerror(PNAMP_ERR_SMALL_NORM));
    return 0;
}
