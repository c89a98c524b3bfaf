/* rl_oracle.h -- CPU FP64 restatement of RADLite's line raytrace (test infrastructure only). */
#ifndef RL_ORACLE_H
#define RL_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct rlo_model rlo_model;
const char* rlo_last_error(void);
int rlo_load_dir(const char* dir, rlo_model** out);
void rlo_free(rlo_model* m);
int rlo_info(const rlo_model* m, int* info, double* dinfo);
int rlo_rays(const rlo_model* m, double* x0, double* z0, double* rays_r, double* ri);
int rlo_trajectory(const rlo_model* m, int iray, int maxn, double* s, double* r, double* th, double* mu,
                   double* phi, int* icr, int* ir, int* it);
int rlo_ray_spectrum(rlo_model* m, int iline, double x0, double z0, double* I_out, double* tau_out);
int rlo_line_image(rlo_model* m, int iline, int ray_begin, int ray_end, double* image, unsigned char* mask,
                   long long* counts);
int rlo_image_to_spectrum(const rlo_model* m, const double* image, double* flux);
int rlo_line_spectrum(rlo_model* m, int iline, double* flux, double* velo_kms, long long* counts);
int rlo_pv_request(const rlo_model* m, int* iv, double* dv);
int rlo_pv_rays(const rlo_model* m, int nx, int ny, double szx, double szy, double phioff, double xoff, double yoff,
                int addstar, double* x0, double* z0, double* b, int* info, double* dinfo);
int rlo_posvel(rlo_model* m, int iline, int nx, int ny, double szx, double szy, double phioff, double xoff,
               double yoff, int addstar, double* I, double* tau);
int rlo_run_dir(const char* dir);
/* bracketing search of the trajectory builder (hunt's index rules) on xx[0..n-1] as 1..n */
int rlo_hunt(const double* xx, int n, double x, int guess);
/* 1 when the last line image, line spectrum or position-velocity cube met the masing
   test of charintline (telescope.F:4291-4297) */
int rlo_masing(const rlo_model* m);
/* formal-solution steps of the last line image, line spectrum or position-velocity cube
   whose quadrature, before the bracket, exceeded twice the theoretical maximum
   (transerr_overshoot, transfer.F:1548-1553) */
long long rlo_overshoots(const rlo_model* m);
#ifdef __cplusplus
}
#endif
#endif
