/* Stand-in for METIS 4's metis.h, used ONLY to compile the reference's
 * meshFIM3dEikonal.cu / meshFIM2d_eikonal.cu for pinning their host set-up.  The
 * pins never partition through it: ref_tethost3d.cu defines the function as a stub
 * that reports failure. */
#pragma once
void METIS_PartGraphKway(int* nvtxs, int* xadj, int* adjncy, int* vwgt, int* adjwgt, int* wgtflag, int* numflag,
                         int* nparts, int* options, int* edgecut, int* part);
