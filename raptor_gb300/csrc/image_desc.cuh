// Per-image constants as the ray kernels see them.  Built on the host in
// FP64 from a raptor_image_desc and its grid (camera set-up of
// metric.c:650-727 and BL_to_KS_u GRmath.c:135-184 that is common to all
// pixels, set_units grmhd.c:17-33, set_constants utilities.c:17-26).
#pragma once
#include "checked.cuh"
#include "kerr_mks.cuh"

namespace raptor {

constexpr int kMaxFreqs = 8;
constexpr double kRcam = 1.e4;                 // parameters.h:163
constexpr double kCutoffOuter = kRcam * 1.01;  // parameters.h:184
constexpr int kMaxOrder = 100;                 // parameters.h:170
constexpr double kMaxSteps = 1e5;              // parameters.h:182
constexpr double kSourceDist = 2.6228263e22;   // parameters.h:144, cm
constexpr double kTwoPi = 6.283185307179586;   // 2.0 * M_PI, exact
constexpr int kCamLog = 1;                     // RAPTOR_CAM_LOG

// cgs constants, constants.h:16-29 and j_nu.c:15
constexpr double kECharge = 4.8032068e-10;
constexpr double kEMass = 9.1093826e-28;
constexpr double kPMass = 1.67262171e-24;
constexpr double kBoltz = 1.3806505e-16;
constexpr double kC = 2.99792458e10;
constexpr double kPlanck = 6.6260693e-27;
constexpr double kGGrav = 6.6742e-8;
constexpr double kE2C = 7.695589048e-30;
constexpr double kE2CH = 1.161410e-03;

constexpr int kEmissionThermal = 0;  // RAPTOR_EMISSION_THERMAL
constexpr int kEmissionKappa = 1;    // RAPTOR_EMISSION_KAPPA
constexpr double kKappa = 3.5;       // j_nu.c:35, 62

// The kappa-distribution fits' constants for one image (host, FP64; see
// kappa.cuh and build_dev_image).
struct KappaConst {
    double ln_jlow, ln_jhigh;  // ln of the X-independent factors of J_low, J_high
    double xj;                 // the emissivity's blend exponent 3 kappa^-3/2
    double ln_alow, ln_ahigh;  // ln of the X- and Theta_e-independent factors of A_low, A_high
    double xa;                 // the absorptivity's blend exponent (-7/4 + 8 kappa/5)^(-43/50)
    double g1, g2;             // the connection formula's gamma-function ratios
};
// the same in FP32, for the FP32 samples of the mixed forms
struct KappaConstF {
    float ln_jlow, ln_jhigh, xj, ln_alow, ln_ahigh, xa, g1, g2;
};

struct DevImage {
    long long ray_begin;   // first global ray of this image
    long long out_offset;  // first double of this image in the output
    int width, height, nfreq, integrator;
    // grid: cells [n1][n2][8], primitives interleaved per cell
    const double* cells64;
    const float* cells32;
    int n1, n2;
    double startx1, startx2, stopx1, stopx2, idx1, idx2;
    Geo geo;
    // camera (integrator.c:188-191, metric.c:652-692)
    double stepx, stepy, half_x, half_y;
    double sin_mu, mu0sq, cc_over_sc, cosc2;
    double g11, gu00, gu03, gu33, gu22;  // BL metric at the camera
    double t01, t31;                     // BL -> KS transform at the camera
    double k2fac;                        // d theta / d x2 at the camera's x2
    double xcam[4];                      // MKS camera position
    // model
    double stepsize, inv_stepsize, cutoff_inner;
    double Ne_unit, B_unit, inv_B_unit, r_high, r_low;
    double freq[kMaxFreqs];
    double nu3[kMaxFreqs];        // freq^3 (core.c:136)
    double rg_over_nu[kMaxFreqs]; // R_g / freq (radiative_transfer.c:88)
    double inv_freq2[kMaxFreqs];  // 1 / freq^2
    // log-polar camera (integrator.c:191-198, core.c:123-133)
    int camera;                   // 0 linear, 1 log-polar
    double ln20;                  // log(20.)
    double rgrav;                 // R_GRAV, cm (utilities.c:20)
    double dtheta_px;             // R_GRAV 2 pi / H
    double dist2;                 // source_dist^2 (parameters.h:144)
    // FP32 copies of the transfer sample's constants (mixed forms)
    float ne_unit_f, b_unit_f, inv_b_unit_f, r_high_f, r_low_f;
    float freq_f[kMaxFreqs], rg_over_nu_f[kMaxFreqs];
    // DF copies of the geodesic's constants (mixed-DF form)
    GeoDF geo_df;
    DF inv_stepsize_df, cutoff_inner_df;
    DF startx1_df, startx2_df, stopx1_df, stopx2_df, idx1_df, idx2_df;
    // the checked build's bounds (checked.cuh): one past the batch's last
    // output double, and the word a failed check is recorded in
    long long out_end;
    unsigned long long* check_word;
    // emission model: kEmissionThermal, or kEmissionKappa with its constants
    int emission;
    KappaConst kap;
    KappaConstF kapf;
    // the point quantities at the camera position xcam, where every ray of
    // the image starts: written by camera_point_kernel (ray_kernel.cuh) on
    // the device after each upload, read by the FP64 and mixed kernels'
    // start_ray
    MksPoint cam_point;
};

// Per-step record of one traced ray (the analogue of the reference's GEOD
// switch, integrator.c:172-240): y[8], d lambda, tau_0, raw I_0, steps,
// theta turns, event (0 no transfer, 1 sigma cut, 2 sampled, 3 escaped),
// stop flag, 0.
constexpr int kTraceWidth = 16;
struct TraceSpec {
    long long ray;  // global ray index to record, or -1
    double* out;    // [cap][kTraceWidth]
    int cap;
};

}  // namespace raptor
