// The legacy entry points' bodies, called by both the C-linkage names
// (voce_legacy.cpp) and the C++-linkage names (voce_legacy_cxx.cpp).
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

void voce_legacy_setup(void);
void voce_legacy_evolution(void);
void voce_legacy_destroy(void);
void voce_legacy_chg_basis(double *V6, double (*T2)[3], double (*C2)[6], double (*T4)[3][3][3], int opt);
void voce_legacy_euler(double *t1, double *ph, double *t2, double (*a)[3], int opt);

#ifdef __cplusplus
}
#endif
