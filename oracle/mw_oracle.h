/* mw_oracle.h -- CPU restatement of the PyMiniWeather time step (test
 * infrastructure; see mw_oracle.c).  All arrays are FP64, C order:
 * state (4, nz+4, nx+4), cell backgrounds (nz+4), interface backgrounds (nz+1). */
#ifndef MW_ORACLE_H
#define MW_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

enum { MWO_DIR_X = 0, MWO_DIR_Z = 1 };
enum { MWO_BG_CONST_THETA = 0, MWO_BG_BVFREQ = 1 };

int mwo_max_threads(void);
void mwo_set_threads(int n);
void mwo_init(int nx, int nz, double xlen, double zlen, int bg, double u0, int nbubble, const double* bubbles,
              double* state, double* hy_dens_cell, double* hy_dens_theta_cell, double* hy_dens_int,
              double* hy_dens_theta_int, double* hy_pressure_int);
void mwo_gravity_source(int nx, int nz, double xlen, double zlen, const double* hy_dens_cell, double* src);
void mwo_dirstage(int nx, int nz, double dx, double dz, double dt_full, const double* hyc, const double* hytc,
                  const double* hyi, const double* hyti, const double* hypi, const double* src_w,
                  const double* init, double* forcing, double* out, double dt_stage, int dir);
void mwo_evolve(int nx, int nz, double dx, double dz, double dt, const double* hyc, const double* hytc,
                const double* hyi, const double* hyti, const double* hypi, const double* src_w, double* state,
                double* state_tmp, int nsteps, int* reverse);
void mwo_stats(int nx, int nz, double dx, double dz, const double* hyc, const double* hytc, const double* state,
               double* mass_energy);

#ifdef __cplusplus
}
#endif
#endif
