// rl_host.h -- host-side model of one RADLite working directory.
#pragma once
#include <string>
#include <vector>

namespace rl {

// The rectangular image request of linespectrum.inp command 2 (telescope.F:190-218).
struct PVSpec {
  int nx = 0, ny = 0;
  double szimx = 0.0, szimy = 0.0;   // full image size [cm]
  double phioff = 0.0, xoff = 0.0, yoff = 0.0;
  int addstar = 0;
  int sizespec = 1;                   // linespectrum.inp size specifier (0: arcsec, read as cm)
};

// Everything the line raytrace reads from the reference's input files.
struct Model {
  // spatial grid: R(ix) = R[ix+1] (ix=-1..nr+2), TH(iy) = TH[iy+1] (iy=-1..ny+2)
  int nr = 0, nth = 0, ny = 0;
  std::vector<double> R, TH;
  // cells of the stored (upper) half, index (ir-1)*nth + (it-1)
  std::vector<double> rho, abun, lw, vel;   // vel: 3 per cell (v_r, v_theta, v_phi) [cm/s]
  int nspec = 0;
  std::vector<int> nsize;                   // sizes per species
  std::vector<double> drho;                 // [spec][cell]
  std::vector<double> dtemp;                // [spec][4][cell]
  int ncont = 0;                            // frequency.inp
  std::vector<double> cnu;                  // [ncont]
  std::vector<double> kabs, ksca;           // [spec][4][ncont]
  std::vector<double> scat;                 // [ncont][cell] (empty if absent)
  int nlev = 0;
  std::vector<double> pop;                  // [cell][nlev]
  // molecule
  std::string molname, molfile;
  std::vector<double> Ecm, gdeg;            // [nlev_mol]
  std::vector<int> lup, ldn;                // 1-based level indices per line
  std::vector<double> Aud, lfreq;           // per line
  double umass = 2.3;
  // star and boundaries
  double rstar = 0.0;
  std::vector<double> starcont;             // intensity at the stellar surface on cnu
  std::vector<double> isrf;                 // interstellar field on cnu (outer boundary 3)
  int starpump = 0, outer_bc = 0, line_dust = 1;
  // camera and passband (radlite.inp, linespectrum.inp)
  double incl_rad = 0.0;
  int nphi = 0, dbdr = 1, nrext = 0;
  double vmax = 0.0, dv = 0.0, radvelo = 0.0;
  int nlspec = 0, ilstart = 1, style = 1, nfr = 0;
  int command = 0;                          // 0: line spectrum, 2: position-velocity cube
  PVSpec pv;
  double aksmax = 0.0;
  int ncell() const { return nr * nth; }
};

// The reference's camera: the circular-image ray family (telescope.F:715-1191).
struct Camera {
  double incl_rad = 0.0;   // after the small-angle clamp
  double theta0 = 0.0;
  int nphi = 0, nrr = 0, nrays = 0;
  std::vector<double> x0, z0;   // [nrays], ray 0 = central beam
  std::vector<double> rays_r;   // [nrr+1]
  std::vector<double> ri;       // [nrr+2] ring edges
};

// The rectangular camera (setup_rays_rectang, telescope.F:2229-2475): pixel rays in the
// reference's order (ix outer, iy inner), then the central ray when the star is added.
struct PVCamera {
  int nx = 0, ny = 0, nrays = 0;
  double spx = 0.0, spy = 0.0, incl_rad = 0.0, theta0 = 0.0;
  int starunres = 0;            // add the unresolved star to the four central pixels
  double srat = 0.0;            // pi R*^2 / (4 spx spy)
  double rmax = 0.0;            // outer grid radius: pixels with b >= 0.999 rmax are empty
  std::vector<double> x0, z0;   // [nrays]
  std::vector<double> b;        // [nx*ny] impact parameter
};

// Per-line constants and cell tables (line.F:427-545, 1708-1823, 3502-3677, 3797-3845).
struct LinePrep {
  double lfreq = 0.0, nu0 = 0.0, Bud = 0.0, Bdu = 0.0, scale = 1.0, istart = 0.0, cphi = 0.0;
  std::vector<double> dnu, velo, wch, star;    // [nfr]
  std::vector<double> isrf;                    // [nfr] outer-boundary start per channel (type 3), else empty
  bool mase = false;                           // some cell has a negative line opacity (inversion)
  std::vector<double> tab;                     // [ncell][4] jfac/scale, afac, jd/scale, ad
  std::vector<double> nsum;                    // [ncell]
};

// Parse the input files of `dir` (or read their binary cache, see RLGPU_INPUT_CACHE).
int load_dir(const std::string& dir, Model& m, std::string& err);
// 64-bit hash over every member of the model (equal models, equal hashes)
unsigned long long model_checksum(const Model& m);
int setup_camera(const Model& m, double incl_rad, int nphi, int dbdr, int nrext, Camera& cam, std::string& err);
int setup_pv_camera(const Model& m, const PVSpec& spec, double incl_rad, PVCamera& cam, std::string& err);
// with_isrf: build the outer-boundary-3 start table (spectra); the position-velocity path
// never fills it in the reference (calc_write_line_posvel, telescope.F:1828-1924)
int prepare_line(const Model& m, int iline, bool scaled, LinePrep& lp, std::string& err, bool with_isrf = true);
double bplanck(double temp, double nu);                     // setup.F:937-952
int bracket(const std::vector<double>& xx, double x);      // 1-based j with xx[j-1] < x <= xx[j]
void finish_model(Model& m);   // derived quantities (aksmax, passband channel count)
// lineposvelcirc_<molecule>_<iline>.dat, the circular image of a SAVE_IMCIR build
// (telescope.F:1595-1615, 1346-1373; empty for iline > 99). img and mask: [nrays][nfr]
// intensities and integration mask (imcir_cmask, accumulated over the run's lines).
std::string imcir_file_name(const Model& m, int iline);
int write_imcir_file(const std::string& path, const Model& m, const Camera& cam, int iline, const double* img,
                     const unsigned char* mask, std::string& err);
// lineposvel_<molecule>_<iline>.dat (telescope.F:1940-1961; empty for iline > 99)
std::string posvel_file_name(const Model& m, int iline);
// I and tau: [nfr][ny][nx] intensity and optical depth of line iline (1-based)
int write_posvel_file(const std::string& path, const Model& m, const PVCamera& cam, const PVSpec& spec, int iline,
                      const double* I, const double* tau, std::string& err);
int write_spectrum_file(const std::string& path, const Model& m, const Camera& cam,
                        const std::vector<int>& lines, const std::vector<double>& flux, std::string& err);

}  // namespace rl
