/*
  METIS stand-in used only to compile the reference TACS sources into the
  CPU checker library (oracle/_ref).  The checker never partitions or
  reorders, so every entry point aborts if reached.
*/
#ifndef ORACLE_STUB_METIS_H
#define ORACLE_STUB_METIS_H

#define METIS_NOPTIONS 40
#define METIS_OPTION_NUMBERING 17

int METIS_SetDefaultOptions(int *options);
int METIS_PartGraphRecursive(int *nvtxs, int *ncon, int *xadj, int *adjncy,
                             int *vwgt, int *vsize, int *adjwgt, int *nparts,
                             double *tpwgts, double *ubvec, int *options,
                             int *edgecut, int *part);
int METIS_PartGraphKway(int *nvtxs, int *ncon, int *xadj, int *adjncy,
                        int *vwgt, int *vsize, int *adjwgt, int *nparts,
                        double *tpwgts, double *ubvec, int *options,
                        int *edgecut, int *part);
int METIS_NodeND(int *nvtxs, int *xadj, int *adjncy, int *vwgt, int *options,
                 int *perm, int *iperm);

#endif
