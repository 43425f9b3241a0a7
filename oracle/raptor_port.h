/* C restatement of RAPTOR's per-pixel imaging path (TEST INFRASTRUCTURE:
 * the oracle that checks the CUDA engine, and the CPU baseline it is timed
 * against on machines where the reference sources are absent).
 *
 * Every function restates the reference algorithm and cites the reference
 * file:line it follows.  No global state: one port_scene describes a grid
 * plus an image, and rays are traced independently (OpenMP over pixels). */
#ifndef RAPTOR_PORT_H
#define RAPTOR_PORT_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct port_scene {
    /* grid (HARM dump header, raptor_harm_model.c:90-135) */
    int n1, n2;
    double startx1, startx2, dx1, dx2;
    double a, hslope, R0;
    const double *prims; /* [8][n1][n2], HARM primitive order */
    /* camera and model (model.in + argv, core.c:22-42) */
    int width, height;
    double cam_size_x, cam_size_y;
    double inclination; /* degrees */
    double stepsize;
    double mbh, m_unit, r_high, r_low;
    int integrator; /* 4 = RK4 (integrator.c:13-41), 2 = RK2 (integrator.c:44-70) */
    int camera;     /* 0 = LINEAR_IMPACT_CAM, 1 = LOG_IMPACT_CAM (parameters.h:54-55) */
    int emission;   /* 0 = the thermal fits emission_coeff calls (j_nu.c:20-26), 1 = the kappa fits (j_nu.c:28-106) */
} port_scene;

typedef struct port_ray_stats {
    int steps;      /* loop iterations of integrate_geodesic */
    int rt_samples; /* radiative_transfer calls that passed get_fluid_params */
    int rt_calls;   /* radiative_transfer calls (in-grid steps) */
    int reason;     /* 1 horizon, 2 escape, 3 outer radius, 4 step cap, 5 theta turns, 6 non-finite */
    double kk;      /* |g_{mu nu} k^mu k^nu| / (k^t)^2 at the last state */
} port_ray_stats;

/* Render the pixels listed in `pixels` (index x + y*width, core.c:108-109)
 * at nfreq frequencies.  out[k*nfreq + f] = I_f * nu_f^3 (core.c:136), or
 * I_f nu_f^3 r_i d_r d_theta / D^2 for the log-polar camera (core.c:123-133).
 * stats may be NULL.  nthreads <= 0 uses all OpenMP threads.  Returns 0. */
int port_render(const port_scene *s, const int *pixels, int n, const double *freqs, int nfreq,
                double *out, port_ray_stats *stats, int nthreads);

/* Per-step records of one ray, the layout of raptor_gpu_trace_ray (16
 * doubles per step, step 0 = initial photon).  Returns records written. */
int port_trace_ray(const port_scene *s, int pixel, const double *freqs, int nfreq, int cap, double *records);

/* Function-level entry points (for known-answer tests). */
void port_metric_dd(const port_scene *s, const double X[4], double g[16]);
void port_metric_uu(const port_scene *s, const double X[4], double g[16]);
void port_connection(const port_scene *s, const double X[4], double G[64]);
void port_init_photon(const port_scene *s, double alpha, double beta, double photon[8]);
double port_camera_x2(const port_scene *s);
double port_j_thsynch(double B, double costh, double thetae, double nu, double ne);
double port_a_th(double j, double nu, double thetae);
double port_hyp2f1(double a, double b, double c, double x);
double port_j_kappa(double nu, double ne, double thetae, double B, double costh);
double port_a_kappa(double nu, double ne, double thetae, double B, double costh);
int port_fluid(const port_scene *s, const double X[4], double out[12]);

#ifdef __cplusplus
}
#endif
#endif
