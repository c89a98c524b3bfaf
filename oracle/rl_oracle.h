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
int rlo_line_image(rlo_model* m, int iline, int ray_begin, int ray_end, double* image, unsigned char* mask,
                   long long* counts);
int rlo_image_to_spectrum(const rlo_model* m, const double* image, double* flux);
int rlo_line_spectrum(rlo_model* m, int iline, double* flux, double* velo_kms, long long* counts);
int rlo_run_dir(const char* dir);
#ifdef __cplusplus
}
#endif
#endif
