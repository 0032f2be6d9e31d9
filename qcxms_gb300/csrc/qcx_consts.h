/* Algorithm constants shared by the CUDA library and the CPU oracle.
 * (Parameters of the Hamiltonian live in qcx_params.h.) */
#ifndef QCX_CONSTS_H
#define QCX_CONSTS_H

/* Boltzmann constant in Hartree/K: src/tblite.f90:43 (ktoau) and
 * src/xtb_mctc_constants.f90:35 (kB) carry the same value. */
#define QCX_KTOAU 3.166808578545117e-06
/* femtoseconds to atomic time units, src/xtb_mctc_convert.f90:54 */
#define QCX_FSTOAU 41.3413733365614

/* Primitive Gaussian pairs with a*b/(a+b)*R^2 above this bound are skipped:
 * their contribution is below exp(-40) ~ 4e-18 of a normalised integral. */
#define QCX_PRIM_SCREEN 40.0

/* SCC defaults. The iteration limit is the one of the xtb programs (250, the
 * default of tblite's calculator), which QCxMS's call keeps (src/tblite.f90:
 * 136 passes no limit); a molecule that needs more fails its energy call. */
#define QCX_SCC_MAXITER 250
#define QCX_SCC_ECONV 1.0e-7
#define QCX_SCC_PCONV 1.0e-6
#define QCX_BROYDEN_ALPHA 0.25
#define QCX_BROYDEN_W0 0.01
/* Broyden history: the last QCX_BROYDEN_WINDOW iterations */
#ifndef QCX_BROYDEN_WINDOW
#define QCX_BROYDEN_WINDOW 24
#endif
/* The mixer restarts (history dropped, the next update a linear mixing step
 * from the current input) when the moment residual has not fallen below 0.9
 * of its best value for this many iterations: charge sloshing between
 * near-degenerate states can hold a Broyden history at a residual of ~3e-2
 * for tens of iterations. */
#ifndef QCX_BROYDEN_RESTART
#define QCX_BROYDEN_RESTART 12
#endif

/* Fermi level bisection: fixed iteration count for reproducibility */
#define QCX_FERMI_ITERS 200

#define QCX_PI 3.14159265358979323846
#endif
