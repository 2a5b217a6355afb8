// C++-linkage names of the legacy entry points: the reference's Makefile
// builds evp.c and io.c with mpicxx, so their calls bind these (the parameter
// types are those of evp.h:21-26, so the names mangle alike).
#include "voce_legacy_impl.h"

typedef double real;
typedef real ten2nd[3][3];
typedef real ten4th[3][3][3][3];
typedef real voigt[6];
typedef real voigt66[6][6];

void SetupJob(void) { voce_legacy_setup(); }
void Evolution(void) { voce_legacy_evolution(); }
void DestroyJob(void) { voce_legacy_destroy(); }
void chg_basis(voigt V6, ten2nd T2, voigt66 C2, ten4th T4, int opt) { voce_legacy_chg_basis(V6, T2, C2, T4, opt); }
void EulerToTransMatrix(real *t1, real *ph, real *t2, ten2nd a, int opt) { voce_legacy_euler(t1, ph, t2, a, opt); }
