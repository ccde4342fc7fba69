/*
  Stand-in for the METIS interface, used only to compile the reference
  sources into the CPU checker under oracle/_ref.  On one rank with natural
  or AMD ordering the reference never partitions, so every entry point
  reports and aborts if it is reached.
*/
#ifndef A2DS_ORACLE_METIS_STUB_H
#define A2DS_ORACLE_METIS_STUB_H
#include <stdio.h>
#include <stdlib.h>

#define METIS_NOPTIONS 40
#define METIS_OPTION_NUMBERING 17

static inline int a2ds_metis_unreachable(const char *f) {
  fprintf(stderr, "%s is not available in the single-process checker\n", f);
  abort();
  return 0;
}
static inline int METIS_SetDefaultOptions(int *options) {
  for (int i = 0; i < METIS_NOPTIONS; i++) options[i] = -1;
  return 1;
}
static inline int METIS_PartGraphRecursive(int *, int *, int *, int *, int *,
                                           int *, int *, int *, double *,
                                           double *, int *, int *, int *) {
  return a2ds_metis_unreachable("METIS_PartGraphRecursive");
}
static inline int METIS_PartGraphKway(int *, int *, int *, int *, int *, int *,
                                      int *, int *, double *, double *, int *,
                                      int *, int *) {
  return a2ds_metis_unreachable("METIS_PartGraphKway");
}
static inline int METIS_NodeND(int *, int *, int *, int *, int *, int *,
                               int *) {
  return a2ds_metis_unreachable("METIS_NodeND");
}
#endif
