/*
 * rlgpu.h -- C ABI of the GB300 line raytrace, a drop-in for RADLite's raytrace step.
 *
 * Reference interfaces replaced (RADLITE/ of pontoppi/radlite):
 *   - the process/file boundary: the RADlite executable run in a directory holding the
 *     input files, writing linespectrum_<mol>.dat and radlite.success
 *     (main.F:26-71; drivers pyradlite/pyradlite/radlite.py:592-595, PRO/line_run.pro:173)
 *     -> rl_run_dir()
 *   - the in-process per-line call `call calc_line_spectrum(iln, linespec_distance,
 *     main_passbwidth, main_passbnfr)` (main.F:1043-1049, telescope.F:1465-1654), whose
 *     result is the COMMON array spec_flux_observer(1:nfr) (telescope.F:1433)
 *     -> rl_line_spectrum() / rl_spectra()
 *   - the input readers (setup.F, grid.F, dust.F, star.F, line.F readers)
 *     -> rl_load_dir(); in-memory arrays of the same content -> rl_load_arrays()
 *   - the circular image (imcir_int, telescope.F:339-631; SAVE_IMCIR dump
 *     telescope.F:1348-1373) -> rl_line_image()
 *
 * Conventions: every call returns 0 on success and a negative code on failure, with a
 * message available from rl_last_error(); the library never exits the process. Buffers
 * are owned by the caller and live in host memory; device memory is owned by the library
 * behind the opaque handles. A handle is used by one host thread at a time.
 */
#ifndef RLGPU_H
#define RLGPU_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rl_ctx rl_ctx;
typedef struct rl_model rl_model;

enum { RL_OK = 0, RL_ERR_ARG = -1, RL_ERR_IO = -2, RL_ERR_CUDA = -3, RL_ERR_GEOMETRY = -4, RL_ERR_STATE = -5 };
enum { RL_FP32 = 0, RL_FP64 = 1 };

typedef struct rl_stats {
  unsigned long long steps;        /* formal-solution steps incl. sub-steps (qdr_src_2 calls) */
  unsigned long long integrated;   /* (ray, channel, line) triples integrated */
  unsigned long long node_visits;  /* integrated triples x nodes of their ray */
  unsigned long long ray_channels; /* rays x channels x lines written to the image */
  double geometry_ms, walk_ms, reduce_ms, upload_ms, total_ms;
  int nrays, nfr, kmax, nlines;
  unsigned long long h2d_bytes, d2h_bytes;   /* host<->device copies made by the call */
  unsigned long long node_passes;    /* walk: a tile's channel slots taken over one node */
  unsigned long long packed_passes;  /* of them on the packed FP32 path (positive opacity,
                                        no state reset, no SUBGRID refinement) */
  unsigned long long empty_steps;    /* steps counted in `steps` whose two nodes have zero
                                        emissivity and opacity: the intensity passes
                                        unchanged and no arithmetic is done */
  unsigned long long refined_passes; /* node passes in which some channel needed SUBGRID
                                        refinement (line.F:4733-4742) */
  unsigned long long sub_steps;      /* steps counted in `steps` that refined channels take
                                        inside such segments */
  unsigned long long refined_channels; /* (channel, segment) pairs refined in those passes */
  unsigned long long overshoots;     /* steps counted in `steps` whose quadrature before the
                                        bracket exceeded twice the theoretical maximum
                                        (transerr_overshoot, transfer.F:1548-1553); counted
                                        with RL_CHECK_OVERSHOOT set (rl_set_checks), by
                                        position-velocity cubes and by rl_run_dir; 0 otherwise */
} rl_stats;

typedef struct rl_model_info {
  int nr, nth, nlev, nlines_mol, nlines_spec, ilinestart, nfr, nphi, dbdr, nrrayextra, nrays, nrings;
  int outer_bc, starpump, line_dust, precision;
  double incl_deg, vmax, dv, rstar, aksmax;
} rl_model_info;

/* In-memory model: the content of the input files as arrays (cgs units as in the files).
   Cell arrays are indexed (ir-1)*nth + (it-1) over the stored upper half of the grid. */
typedef struct rl_model_arrays {
  int nr, nth;
  const double* radius;     /* [nr]   radius.inp */
  const double* theta;      /* [nth]  theta.inp (0 .. pi/2, mirrored about the equator) */
  const double* rho;        /* [ncell] gas density (density.inp) */
  const double* abund;      /* [ncell] molecular abundance (abundance.inp) */
  const double* width;      /* [ncell] local line width [km/s] (turbulence.inp) */
  const double* vel;        /* [ncell*3] v_r, v_theta, v_phi [cm/s] (velocity.inp) */
  int nlev;
  const double* pop;        /* [ncell*nlev] level populations (levelpop_<mol>.dat) */
  int nlines_mol;
  const int* lev_up;        /* [nlines_mol] 1-based (moldata.dat) */
  const int* lev_low;
  const double* aud;        /* [nlines_mol] Einstein A [1/s] */
  const double* energy_cm;  /* [nlev] level energies [1/cm] */
  const double* gdeg;       /* [nlev] statistical weights */
  double umass;             /* mean molecular weight (line.inp) */
  int line_dust;            /* include dust in the lines (radlite.inp) */
  int ncont;                /* frequency.inp */
  const double* freq;       /* [ncont] */
  const double* dust_rho;   /* [ncell] one species, one size (dustdens.inp) */
  const double* dust_temp;  /* [ncell] (dusttemp_final.dat) */
  const double* kappa_abs;  /* [ncont] (dustopac_1.inp) */
  const double* kappa_scat; /* [ncont] */
  double rstar;             /* starinfo.inp [cm] */
  const double* star_flux_1pc; /* [ncont] F_nu at 1 pc (starspectrum.inp) or NULL (no star pumping) */
  int outer_bc;             /* 0 black, 2 microwave background (3, the interstellar field of
                               interstellfield.inp, only through rl_load_dir) */
  double incl_deg;          /* linespectrum.inp */
  int nphi, dbdr, nrrayextra;  /* radlite.inp circular image */
  double vmax, dv, radvelo; /* passband half width, sampling, radial velocity [km/s] */
  int ilinestart, nlines_spec;
  const char* molname;      /* output file tag: linespectrum_<molname>.dat */
} rl_model_arrays;

int rl_create(rl_ctx** ctx, int device);
/* Models, batches and differentiable handles made on a context must be released before
   the context itself. */
int rl_destroy(rl_ctx* ctx);
/* Copies the last error message of the context (or of the process for a NULL context). */
int rl_last_error(rl_ctx* ctx, char* buf, size_t len);

int rl_load_dir(rl_ctx* ctx, const char* dir, rl_model** model);
int rl_load_arrays(rl_ctx* ctx, const rl_model_arrays* arrays, rl_model** model);
int rl_model_free(rl_model* model);
/* 64-bit hash of everything the model holds from its inputs (inspection and tests; no
   reference counterpart). Input cache: with the environment variable RLGPU_INPUT_CACHE
   naming a writable directory, rl_load_dir keeps each parsed directory there in binary,
   keyed by its real path and the size and modification time of every input file the
   parse opened or probed, and reads that binary while the files are unchanged. */
int rl_model_checksum(rl_model* model, unsigned long long* checksum);
int rl_model_get_info(rl_model* model, rl_model_info* info);

/* Camera override (radlite.inp / linespectrum.inp values are the default). */
int rl_set_camera(rl_model* model, double incl_deg, int nphi, int dbdr, int nrrayextra);
/* RL_FP32 (default): FP64 geometry, FP32 transfer. RL_FP64: FP64 throughout. */
int rl_set_precision(rl_model* model, int precision);
/* Diagnostics of the model's own line renders (spectra, images, image rows), off by default;
   batches (rl_batch_*) and the differentiable path (rl_diff_*) do not take them.
   RL_CHECK_OVERSHOOT: take the reference's overshoot test on every formal-solution step,
   the check its default build compiles in (transfer.F:1548-1553, not SRCQDR_NO_ERRCHECK),
   and count the steps that fail it in rl_stats.overshoots. The results are unchanged; the
   FP32 walk takes about 10% longer (13.1 -> 14.4 ms on a 400x200 band disk of 20 lines). */
#define RL_CHECK_OVERSHOOT 1
int rl_set_checks(rl_model* model, int flags);

/* F_nu at 1 pc of line `iline` (1-based line of moldata.dat), channel order of the
   passband (ascending frequency), like spec_flux_observer after calc_line_spectrum.
   velo_out (may be NULL) receives the output-file velocities [km/s]. */
int rl_line_spectrum(rl_model* model, int iline, double* flux_out, double* velo_out, rl_stats* stats);
/* Lines iline0 .. iline0+nlines-1 in one launch; flux_out is [nlines][nfr]. */
int rl_spectra(rl_model* model, int iline0, int nlines, double* flux_out, rl_stats* stats);
/* Circular image of one line: [nrays][nfr] intensities (ray 0 = central beam, then
   rings from the inside out, azimuth fastest), as imcir_int. */
int rl_line_image(rl_model* model, int iline, double* image_out, rl_stats* stats);
/* Lines iline0 .. iline0+nlines-1 in one launch, as rl_spectra (flux_out [nlines][nfr],
   may be NULL), also returning the image rows of `nsel` chosen rays: rows_out
   [nlines][nsel][nfr] holds imcir_int(:, iphi, iring) of rays[i] (ray numbering of
   rl_line_image), gathered on the device. A ray sample of the circular image of
   telescope.F:339-631 without reading back the whole image; ray indices outside the
   camera are rejected. */
int rl_image_rows(rl_model* model, int iline0, int nlines, int nsel, const int* rays, double* flux_out,
                  double* rows_out, rl_stats* stats);
/* The same image and its integration mask [nrays][nfr]: 1 where the channel was integrated
   as channel 1 or inside the ray's velocity window (imcir_cmask, telescope.F:548,575), 0
   where it holds the ray's continuum. */
int rl_line_image_mask(rl_model* model, int iline, double* image_out, unsigned char* mask_out, rl_stats* stats);
/* 1 in *detected when the last render of line iline (spectrum, image or position-velocity
   cube of this model) integrated a segment whose line opacity at its end times its length
   is below -0.01, the masing test of charintline (telescope.F:4291-4297), after which the
   reference prints "WARNING: Masing detected!"; else 0. Only lines with a population
   inversion somewhere are tested (the batch reports its own with rl_batch_job_masing; the
   differentiable path's LTE populations have no inversion). */
int rl_line_masing(rl_model* model, int iline, int* detected);

/* ---- Position-velocity cube (linespectrum.inp command 2): the rectangular image of
   setup_rays_rectang / make_freq_image_rectang / calc_write_line_posvel
   (telescope.F:1828-2475). The request is read from a command-2 linespectrum.inp by
   rl_load_dir, or set here; the camera inclination is the model's (rl_set_camera). */
typedef struct rl_posvel_spec {
  int nx, ny;                  /* pixels, both even (imr_nx, imr_ny) */
  double szimx, szimy;         /* full image size [cm] as in the file (size specifier 1) */
  double phioff;               /* image rotation [rad] */
  double xoff, yoff;           /* image offsets [cm] */
  int addstar;                 /* > 0: add the unresolved star to the four central pixels */
} rl_posvel_spec;
int rl_set_posvel(rl_model* model, const rl_posvel_spec* spec);
int rl_get_posvel(rl_model* model, rl_posvel_spec* spec);
/* Lines iline0 .. iline0+nlines-1: I_out and tau_out (either may be NULL) receive
   [nlines][nfr][ny][nx] intensity [erg/s/cm^2/Hz/ster] and line-of-sight optical depth,
   as imrec_int and imrec_tau (per channel, iy outer, ix inner: the file's order). */
int rl_posvel(rl_model* model, int iline0, int nlines, double* I_out, double* tau_out, rl_stats* stats);

/* ---- Spectrum post-processing: pyradlite's RadliteSpectrum.gen_spec numerical core
   (_process_spectrum, pyradlite/radlite.py:3001-3187). The caller reads and de-duplicates
   the lines (radlite.py:2750-2998); this combines them into one observed spectrum. */
typedef struct rl_genspec_lines {
  int nlines;
  const int* npts;            /* [nlines] channels of each line */
  const double* vel;          /* concatenated velocities [km/s], ascending within a line */
  const double* flux;         /* concatenated F_nu at 1 pc [erg/s/cm^2/Hz] */
  const double* freq;         /* [nlines] line centre [Hz] */
  const int* maxnumpoints;    /* [nlines] channel count of the line's output file */
} rl_genspec_lines;
typedef struct rl_genspec_params {
  double obsres;              /* observing resolution (kernel width) [km/s] */
  double vsampling;           /* output sampling [km/s] */
  double dist;                /* distance [pc] */
} rl_genspec_params;
/* Number of output points (the wavelength grid of the result). */
int rl_gen_spec_size(const rl_genspec_lines* lines, const rl_genspec_params* params, long long* nout);
/* wavelength [micron], frequency [Hz], spectrum / emission / continuum [Jy at dist]:
   [nout] each. Fails like the reference where its interpolations would leave their
   range (an output grid reaching beyond the fine grid). */
int rl_gen_spec(rl_ctx* ctx, const rl_genspec_lines* lines, const rl_genspec_params* params, double* wavelength,
                double* frequency, double* spectrum, double* emission, double* continuum, rl_stats* stats);

/* The RADlite executable's work in `dir`: read the inputs and render the lines requested
   by linespectrum.inp (starting at line 1, main.F:204). Command 0 writes
   linespectrum_<mol>.dat (main.F:1034-1049), command 2 one lineposvel_<mol>_<iline>.dat
   per line (main.F:1061-1074); both then write radlite.success. The run takes the
   overshoot test on every step (RL_CHECK_OVERSHOOT) and, like the reference, appends the
   run's record to radlite.log: the start stamp, this build's switches and the problem
   setup before the render, the warnings (the overshoot warning of main.F:1547-1552 when a
   step failed the test) and the finish stamp after it (write_logmessage_start/_end,
   main.F:1121-1588). */
int rl_run_dir(const char* dir, int device, rl_stats* stats);
/* rl_run_dir with options. RL_RUN_SAVE_IMCIR: as a reference build with SAVE_IMCIR
   (configure_image.h:57), also write lineposvelcirc_<mol>_<iline>.dat, the circular image
   and integration mask of every line of a command-0 run (telescope.F:1346-1373). */
#define RL_RUN_SAVE_IMCIR 1
int rl_run_dir_ex(const char* dir, int device, int flags, rl_stats* stats);

/* Node list of one ray as the geometry kernel produces it (inspection and tests):
   returns the node count (may exceed cap; arrays receive min(count, cap) entries). */
int rl_debug_trajectory(rl_model* model, int iray, int cap, double* s, double* r, double* theta, double* mu,
                        double* dvmu, int* icr, int* ir, int* it);

/* Measured throughput of the two pipes that bound the formal solution: FP32 FFMA
   instructions per second (lane operations) and MUFU ex2 operations per second over the
   whole device. Roofline denominators; no counterpart in the reference. */
int rl_measure_peaks(rl_ctx* ctx, double* ffma_per_s, double* ex2_per_s);

/* ---- Batched rendering: many (model, camera, line range) jobs in one launch sequence.
   Replaces the drivers' one-process-per-model loop (pyradlite radlite.py:592-595, IDL
   line_run.pro:173) and the per-line calc_line_spectrum loop (main.F:1043-1049) with one
   geometry launch, one persistent walk fed from a device work queue and one reduction per
   memory wave, captured once in a CUDA graph and replayed. A job snapshots its model's
   camera at the first run; models must outlive the batch and keep their grid. */
typedef struct rl_batch rl_batch;
int rl_batch_create(rl_ctx* ctx, int precision, rl_batch** batch);
int rl_batch_destroy(rl_batch* batch);
/* Adds lines iline0 .. iline0+nlines-1 of `model` at its current camera; returns the job
   index (>= 0). */
int rl_batch_add(rl_batch* batch, rl_model* model, int iline0, int nlines);
/* Device bytes per memory wave (node records, images, ring sums); 0 = 70% of free memory. */
int rl_batch_set_memory(rl_batch* batch, double bytes);
/* Tile shape of the walk: lines per work item (1..32; a warp walks the item's (line,
   channel) pairs in tiles of 32 x slots pairs spanning at most 12 lines) and channel slots
   per lane (1, 2, 4, 8). Default 32 lines, 4 slots. */
int rl_batch_set_tiles(rl_batch* batch, int lines_per_item, int channel_slots);
int rl_batch_get_tiles(rl_batch* batch, int* lines_per_item, int* channel_slots);
/* Times the tile shapes (2, 8, 16, 32 lines per item, 4 slots: the walk steps four slots
   per lane together) on every
   sample_stride-th work item of the first wave and keeps the fastest, the default shape
   unless another beats it by 2% (a stride of 8 or less samples enough items to rank them);
   returns it and the sampled walk time. No counterpart in the reference. */
int rl_batch_autotune(rl_batch* batch, int sample_stride, int* lines_per_item, int* channel_slots,
                      double* sample_ms);
/* 1 (default): capture the launch sequence in a CUDA graph at the first run, replay after. */
int rl_batch_use_graph(rl_batch* batch, int enable);
/* Number of flux values (sum over jobs of nlines x nfr) and the layout of one job in them. */
int rl_batch_flux_size(rl_batch* batch, long long* n);
int rl_batch_job_info(rl_batch* batch, int job, long long* flux_offset, int* nlines, int* nfr);
/* Renders every job; flux_out receives each job's [nlines][nfr] F_nu at 1 pc in job order. */
int rl_batch_run(rl_batch* batch, double* flux_out, rl_stats* stats);
/* Masing test of the last run, per line of job `job` (detected[nlines]: 1 where a segment's
   line opacity at its end times its length fell below -0.01, as rl_line_masing reports
   for a model, telescope.F:4291-4297). Only jobs with a population inversion are tested. */
int rl_batch_job_masing(rl_batch* batch, int job, int* detected);
/* Memory waves of the last build. */
int rl_batch_waves(rl_batch* batch, int* nwaves);
/* The executable's work for every directory listed in `manifest` (one per line, '#'
   comments), rendered as one FP32 batch: each directory gets its linespectrum_<mol>.dat
   and radlite.success. Replaces the drivers' one-process-per-directory loop
   (radlite.py:592-595). */
int rl_run_manifest(const char* manifest, int device, rl_stats* stats);

/* ---- Differentiable raytrace. No counterpart in the reference, whose level populations
   come precomputed from the setup (LTE in pyradlite radlite.py:1106-1118). A rl_diff holds
   one model's camera and lines iline0 .. iline0+nlines-1; the spectra become a function of
   three per-cell parameters (cell index (ir-1)*nth + (it-1)): ln T (gas and dust
   temperature; LTE populations with the partition sum over the molecule's levels), ln X
   (molecular abundance) and the line width b [km/s] (turbulence.inp). Everything else stays
   as loaded, including the largest width (velocity-window margin) and the FP32 intensity
   scale. All array arguments are DEVICE pointers of the context's device (FP64); the calls
   return after the work is done. */
typedef struct rl_diff rl_diff;
int rl_diff_create(rl_model* model, int iline0, int nlines, int precision, rl_diff** diff);
int rl_diff_destroy(rl_diff* diff);
int rl_diff_info(rl_diff* diff, int* ncell, int* nlines, int* nfr, int* nrays);
/* How the backward call walks the rays. 0 (the default): the gradient sweep in walk
   order, no stored intensities: the forward also keeps each channel's optical depth along
   the ray (two image-sized buffers), and the backward recomputes every step and takes its
   gradient with the multiplier e^{-(optical depth still ahead)}. 1 or 32: the reverse
   sweep, which keeps the intensity entering every node (1: 32 values a node per resident
   warp, about 0.1-0.4 GB) or every 32nd node (the chunk is walked again). All give the
   same gradient. A change of mode needs a new rl_diff_forward before rl_diff_backward. */
int rl_diff_set_checkpoint(rl_diff* diff, int every);
/* flux [nlines][nfr]: F_nu at 1 pc for the parameters lnT, lnX, width [ncell]. */
int rl_diff_forward(rl_diff* diff, const double* lnT, const double* lnX, const double* width, double* flux,
                    rl_stats* stats);
/* Gradient of a loss L at the last forward's parameters: given gflux = dL/dflux
   [nlines][nfr], writes dL/dlnT, dL/dlnX, dL/dwidth [ncell] (the adjoint walk chosen by
   rl_diff_set_checkpoint). */
int rl_diff_backward(rl_diff* diff, const double* gflux, double* g_lnT, double* g_lnX, double* g_width,
                     rl_stats* stats);

/* Many differentiable models rendered together: one forward launch sequence (LTE tables
   and node widths per model, then one persistent walk over all models' items from a device
   queue and one reduction) and one persistent adjoint launch, each captured once in a CUDA
   graph and replayed. The batch owns concatenated device buffers (FP64): parameters
   ln T, ln X, width [sum of ncell], spectra and their gradient [sum of nlines x nfr],
   parameter gradients [sum of ncell]; rl_diff_batch_layout gives a model's offsets.
   Fill the parameters (and gflux before a backward) in place, then call forward/backward;
   the calls return after the work is done. All models share one precision. */
typedef struct rl_diff_batch rl_diff_batch;
int rl_diff_batch_create(rl_ctx* ctx, rl_diff_batch** batch);
int rl_diff_batch_destroy(rl_diff_batch* batch);
int rl_diff_batch_add(rl_diff_batch* batch, rl_diff* diff);   /* returns the model index */
int rl_diff_batch_use_graph(rl_diff_batch* batch, int enable);
int rl_diff_batch_buffers(rl_diff_batch* batch, double** lnT, double** lnX, double** width, double** flux,
                          double** gflux, double** g_lnT, double** g_lnX, double** g_width, long long* ncell,
                          long long* nflux);
int rl_diff_batch_layout(rl_diff_batch* batch, int model, long long* cell_offset, long long* flux_offset);
int rl_diff_batch_forward(rl_diff_batch* batch, rl_stats* stats);
int rl_diff_batch_backward(rl_diff_batch* batch, rl_stats* stats);

/* Circular image -> F_nu at `distance_pc` parsec, with no device allocation. No
   counterpart in the reference: it serves callers that own all device memory (their
   own pool or arena) and cannot let a library call cudaMalloc. Every pointer is a
   device pointer of the calling thread's current device; `stream` is a cudaStream_t
   (NULL = the default stream); the call only enqueues work on it.
     image  [nlines][nrays][nfr], float (RL_FP32) or double (RL_FP64), ray 0 the
            central beam, then rings from the inside out, azimuth fastest
     ri     [nrr+2] ring edges (ri[1] the central-beam radius), scale [nlines] a factor
            per line, flux [nlines][nfr] output; nrays must be 1 + nrr*nphi.
   The ring sums live in a fixed 8 MiB array in the library's device image (2^20
   doubles, held by every GPU that loads the library until exit); (nrr+1)*nfr above
   2^20 is rejected with RL_ERR_ARG. Nothing in it has to start at zero. Calls that
   overlap on one device (other streams or threads) share that array and race: order
   them on one stream. Every call looks the array's address up on the current device
   (cudaGetSymbolAddress), so a cudaDeviceReset or another current context between calls
   is safe; the first call in a context loads the module: make it before any stream
   capture. Errors: rl_last_error(NULL, ...). */
int rl_image_to_spectrum_noalloc(void* stream, int precision, const void* image, int nlines, int nrays, int nphi,
                                 int nrr, int nfr, const double* ri, const double* scale, double distance_pc,
                                 double* flux);

#ifdef __cplusplus
}
#endif
#endif
