/*
 * yarn_oracle.h -- CPU restatement of the reference's per-step yarn-level
 * cloth solve, used ONLY as a test oracle and as the timed CPU baseline.
 *
 * This is test infrastructure: the GPU product never links, loads or calls
 * it. Every function in yarn_oracle.c names the reference file:line it
 * restates (paths relative to the reference project root).
 *
 * Degrees of freedom follow the reference exactly (src/Cloth.cpp:31-35,
 * src/MatrixMp.cpp:40-99): [x,y,z of every node (node = u + v*W)] followed by
 * [u,v of every interior node (idx = (u-1) + (v-1)*(W-2))].
 */
#ifndef YARN_ORACLE_H
#define YARN_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct yo_cloth yo_cloth;

typedef struct {
  int width, length;          /* nodes along warp (u) and weft (v) */
  double height, L, R;        /* build height, crossing spacing, yarn radius */
  int pose;                   /* 0 = Upright, 1 = Flat (src/Cloth.cpp:57-59) */
  int weave;                  /* 0 = Plain, 1 = Twill, 2 = Satin (src/Cloth.cpp:69-92) */
  /* material per yarn line; Y and B are moduli, ks = Y*PI*R^2, kb = B*PI*R^2
   * (src/Yarn.h:12-16). Warp line index = node row v (length entries), weft
   * line index = node column u (width entries). */
  const double *warp_rho, *warp_Y, *warp_B;
  const double *weft_rho, *weft_Y, *weft_B;
  double kc, kf, df, mu, S, handle_stiffness;
  double G[3];
  double wind_vel[3];
  double wind_density, wind_drag;
  int n_handles;
  const int *handles;         /* n_handles (u,v) pairs */
} yo_desc;

typedef struct {
  long cg_iterations;
  double cg_error;            /* sqrt(|r|^2 / |b|^2) at exit */
  int status;                 /* 0 ok, 1 non-finite A/b/solution */
} yo_stats;

yo_cloth *yo_create(const yo_desc *desc);
void yo_destroy(yo_cloth *c);
int yo_num_nodes(const yo_cloth *c);
int yo_dim(const yo_cloth *c);

/* Node-ordered state arrays (node = u + v*W): lpos/lposfix/lvel [N*3],
 * epos/eposbar/evel [N*2]. set_state refreshes the element geometry
 * (src/Cloth.cpp:421-438 then UpdateClothUnits). */
void yo_set_state(yo_cloth *c, const double *lpos, const double *lposfix, const double *lvel,
                  const double *epos, const double *eposbar, const double *evel);
void yo_get_state(const yo_cloth *c, double *lpos, double *lposfix, double *lvel, double *epos,
                  double *eposbar, double *evel);
void yo_get_normals(const yo_cloth *c, double *normals /* N*3, zero on the boundary */);
void yo_set_wind(yo_cloth *c, const double wind_vel[3]);

/* FillMV (src/PhysicsCloth.cpp:46-156) into the oracle's sparse storage. */
void yo_fill(yo_cloth *c);
/* Dense export of the last yo_fill, reference layout (dim x dim row-major):
 * M = get_SpaM, K = get_SpaFPos, D = get_SpaFVel, F = get_SpaF, V = get_SpaVel,
 * slide = F_E_is_Slides[0] (interior count * 2). Any pointer may be NULL. */
void yo_export_dense(const yo_cloth *c, double *M, double *K, double *D, double *F, double *V,
                     double *slide);
/* Assembled system of the last yo_fill: A = M - h^2 K - h D,
 * b = h (F + ext - D^T V) + M V (src/TrainHelper.cpp:19-20, 63). */
void yo_export_system(const yo_cloth *c, double h, const double *ext_force, double *A, double *b);

/* One SimStep (src/TrainHelper.cpp:15-54 / 56-97): fill, assemble, Jacobi-CG
 * (Eigen ConjugateGradient defaults when cg_tol <= 0 and cg_maxiter < 0),
 * Cloth::update (src/Cloth.cpp:111-148). Returns stats.status. */
int yo_step(yo_cloth *c, double h, const double *ext_force, double cg_tol, long cg_maxiter,
            yo_stats *stats);

/* Plain dense Jacobi-PCG on a caller-provided dense system (restatement of
 * Eigen's ConjugateGradient<..., Lower|Upper> with DiagonalPreconditioner). */
long yo_dense_pcg(int n, const double *A, const double *b, double *x, double tol, long maxiter,
                  double *err_out);

#ifdef __cplusplus
}
#endif
#endif
