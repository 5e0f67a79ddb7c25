/*
 * fdfk_gb300: GB300 (sm_103a) replacement for the hot path of FDFK2D, the
 * hybrid finite-difference / frequency-wavenumber teleseismic solver.
 *
 * The C ABI below is what the reference host (src/FDFK2D.f90) binds through
 * iso_c_binding.  Plain pointers and sizes only; every array uses the
 * reference's Fortran layout (column-major, the index ranges given per
 * argument).  Every function returns FDFK_OK (0) or a negative status and
 * never exits the process; fdfk_last_error() describes the last failure of
 * the calling thread.
 *
 * Grid conventions (src/FDFK2D.f90:125, src/Input.f90:177-183):
 *   NZ = nz + npml - izt + 1 rows (iz = izt..nz+npml; izt = 1 with a free surface
 *   on top, izt = 1 - npml with the absorbing layer on top, is_PML_top)
 *   NX = nx + 2*npml columns (ix = 1-npml..nx+npml)
 *   c(1:3, NZ, NX) = rho, lambda, mu
 *   ux, uz (1:2, NZ, NX): level 1 = u^n, level 2 = u^{n-1}
 *   background strips (12 arrays, time axis 0..nt last), shapes as allocated
 *   in src/FDFK2D.f90:328-355, in the order of the updatedispl_ argument list:
 *   uxl_reg uzl_reg uxr_reg uzr_reg uxb_reg uzb_reg uxl_pml uzl_pml uxr_pml
 *   uzr_pml uxb_pml uzb_pml.
 */
#ifndef FDFK_GB300_H
#define FDFK_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define FDFK_OK 0
#define FDFK_EINVAL (-1)       /* bad argument or inconsistent sizes */
#define FDFK_EUNSUPPORTED (-2) /* a mode this build does not implement */
#define FDFK_ENOMEM (-3)       /* device or host allocation failed */
#define FDFK_ECUDA (-4)        /* a CUDA call failed */
#define FDFK_ESTATE (-5)       /* call out of order (e.g. no background yet) */

/* Scalar arguments of updatedispl_ (src/FDFK2D.f90:516-519), same meaning. */
typedef struct fdfk_params {
    int norder;     /* half FD order, 1..8 */
    int nx, nz;     /* interior grid */
    int npml;       /* absorbing-layer width in cells (>= 2*norder-1) */
    int is_PML_top; /* reference logical: 0 free surface on top (izt = 1), 1 absorbing layer on top
                       (izt = 1 - npml: npml more rows above row 1) */
    int npower;     /* damping profile exponent (reference: 2) */
    int nbd;        /* background-strip width, 2*norder-1 */
    int nt;         /* last time index; strips hold nt+1 samples */
    float dx, dz;
    double dt;
    float vpml;     /* PML reference velocity (reference: max Vp) */
    double R0;      /* target reflection coefficient (reference: 1e-3) */
} fdfk_params;

typedef struct fdfk_session fdfk_session;

/* Library version (major*10000 + minor*100 + patch). */
int fdfk_version(void);

/* Description of the last failure on this thread ("" if none). */
const char* fdfk_last_error(void);

/* Number of step-kernel launches issued by this process so far. */
long long fdfk_kernel_launches(void);

/*
 * Create a solver session on the current CUDA device: allocates the resident
 * wavefield, PML and material state in HBM and uploads c(1:3, NZ, NX).
 * Replaces the allocations of simulate_wavefield (src/FDFK2D.f90:253-306)
 * and the per-call copies of the material into the operators.
 */
int fdfk_session_create(const fdfk_params* p, const float* c, fdfk_session** out);

/* Bind the session to a CUDA stream (cudaStream_t passed as void*; NULL = default).
 * Work already queued on the previous stream is ordered before the new one's. */
int fdfk_session_set_stream(fdfk_session* s, void* stream);

/*
 * Upload background strips for time indices [t0, t0 + count) from the 12
 * host arrays (full reference arrays covering 0..nt).  The strips are what
 * comput_background_wavefield (src/FDFK2D.f90:432-434) produces.
 */
int fdfk_session_upload_background(fdfk_session* s, const float* const strips[12], int t0, int count);

/*
 * Receivers (src/Input.f90:227-249) and the sampling cadence of the time
 * loop (src/FDFK2D.f90:311-315): a sample is taken before the step whenever
 * it == istp*nstp, for istp = 0..nsis.
 */
int fdfk_session_set_receivers(fdfk_session* s, int nrcv, const float* rx, const float* rz, float x0, float z0,
                               int nstp, int nsis);

/*
 * Advance `nsteps` time steps of the loop src/FDFK2D.f90:465-532
 * (receiver sampling + updatedispl_), asynchronously on the session stream.
 * The background for every step must have been uploaded.
 */
int fdfk_session_advance(fdfk_session* s, int nsteps);

/*
 * fdfk_session_advance with a CUDA-event pair around each kernel launch of
 * every sample_every-th step (on the stream that launches it), then a
 * synchronize: *ms_interior is the mean time per launch of the interior
 * fast-path kernel over the sampled steps, *ms_edge that of the tiled kernel
 * (top rows, absorbing layers, receivers), and *ms_total (if not NULL) the
 * time of all nsteps steps between two events on the session's stream, so the
 * kernels' times and the steps' time come from the same loop.  Measurement only.
 */
int fdfk_session_advance_timed(fdfk_session* s, int nsteps, int sample_every, float* ms_interior, float* ms_edge,
                               float* ms_total);

/* Cells per step handled by the interior fast path and by the tiled kernel. */
int fdfk_session_interior_cells(const fdfk_session* s, long long* interior, long long* edge);

/* Time index of the next step (0 after create). */
int fdfk_session_step_index(const fdfk_session* s);

/* Wait for the session stream. */
int fdfk_session_synchronize(fdfk_session* s);

/* Copy the seismograms seisx/seisz(0:nsis, 1:nrcv) to host (radial component before
 * the back-azimuth projection of src/FDFK2D.f90:537-542). */
int fdfk_session_download_seismograms(fdfk_session* s, float* seisx, float* seisz);

/* Copy samples [first, first + count) of every receiver into host arrays of
 * shape (count, nrcv) (sample fastest). */
int fdfk_session_download_seismogram_range(fdfk_session* s, int first, int count, float* seisx, float* seisz);

/*
 * Copy the full time-stepping state between host arrays in the reference
 * layout and the device: ux, uz (1:2, NZ, NX); bp[12] and bu[24] in the
 * updatedispl_ argument order (src/FDFK2D.f90:519-522; the four top-PML bp
 * arrays and six top-PML bu arrays are unused with a free surface and may be
 * NULL).  `it` sets the time index of the next step on upload.
 */
int fdfk_session_upload_state(fdfk_session* s, const float* ux, const float* uz, const float* const bp[12],
                              const float* const bu[24], int it);
int fdfk_session_download_state(fdfk_session* s, float* ux, float* uz, float* const bp[12], float* const bu[24]);

/*
 * Launch shapes of a session (results are identical for every choice): the
 * fast path's segment length in columns (8..1024) and the absorbing-layer
 * tile length along the layer (8..64); 0 keeps the current value.
 */
int fdfk_session_set_tuning(fdfk_session* s, int seg_len, int pml_run);
int fdfk_session_get_tuning(const fdfk_session* s, int* seg_len, int* pml_run);

/*
 * Autotuner: times candidate launch shapes (segment lengths 16..96 and the
 * shortest ones that fill one and two whole waves of fast-path warps;
 * absorbing-layer tile lengths 12..48) for sessions of parameters p and
 * material c on a scratch
 * session (zero state and background, CUDA events; each timed window
 * `steps` steps, or more where that is shorter than 4 ms, up to
 * max(steps, 1000)), re-times the three fastest in three interleaved rounds
 * and returns the winner, for fdfk_session_set_tuning.
 */
int fdfk_autotune(const fdfk_params* p, const float* c, int steps, int* seg_len, int* pml_run, float* ms_per_step);

/*
 * Snapshot of level 2 (u^{n-1} before the next step) of rows 1..nz, columns
 * 1..nx into host arrays (nz, nx), z fastest, as the snapshot files of
 * src/FDFK2D.f90:467-494 hold.  Waits for the session stream.
 */
int fdfk_session_snapshot(fdfk_session* s, float* ux, float* uz);

void fdfk_session_destroy(fdfk_session* s);

/*
 * Receiver functions by iterative time-domain deconvolution, one per trace:
 * the computation of utils/makeRFitdecon.m (called from utils/plot_PRF.m and
 * plot_SRF.m on a solve's seismograms), in FP64 on the GPU, one block per
 * trace.  num (radial for P-to-S) and den (vertical) hold ntr traces of nt
 * samples, trace j at num + j*ld; dt in s; minlag, maxlag, tshift in s (the
 * reference halves minlag / maxlag until the lags fit the trace); f0 the
 * Gaussian width; at most itmax (<= 4096) spikes while the misfit improves by
 * more than minderr (percent).  Writes *nrf, the receiver-function length
 * (it depends only on the lags and tshift); with rf == NULL nothing else is
 * done.  Otherwise rf receives trace j's receiver function at rf + j*ldrf
 * (ldrf >= *nrf), rms the misfit after each iteration at rms + j*itmax and
 * iters the iterations done.  Replaces the MATLAB function
 * makeRFitdecon(UIN, WIN, DT, MINLAG, MAXLAG, TSHIFT, F0, ITMAX, MINDERR, 0)
 * (utils/makeRFitdecon.m:1-3).
 */
int fdfk_rf_itdecon(const float* num, const float* den, int nt, int ntr, int ld, double dt, double minlag,
                    double maxlag, double tshift, double f0, int itmax, double minderr, double* rf, int ldrf,
                    int* nrf, double* rms, int* iters);

/*
 * The input folder of FDFK2D (src/Input.f90): the inpar file names, in
 * order, the FD model, source, receiver, left and right FK model, Vp and Vs
 * model files.  Text files are read with Fortran list-directed rules; the
 * Vp/Vs models are SU files of nx + 2 npml traces (240-byte headers) of
 * nz + npml - izt + 1 samples.  fdfk_input_read fills *in (arrays allocated
 * here, released by fdfk_input_free) and, when write_model_copies is set,
 * writes <model>_without_pml.su next to the input models as the reference
 * does (src/Input.f90:311-321).
 */
typedef struct fdfk_input {
    int norder;                 /* half order, after the reference's reduction to npml */
    int nx, nz, npml, izt;
    int is_PML_top, outsnap, nstep, src_type;
    int nrcv, nlayer_left, nlayer_right;
    int negative_velocity;      /* a negative vp or vs was read (the reference prints an error) */
    float x0, z0, dx, dz, tmax, tstp, f0, ds;
    double dt, rayp;            /* rayp in s/m (read in s/deg) */
    double evla, evlo, lat_org, lon_org, az_org;
    float* rx;
    float* rz;
    float* fk_left;             /* (4, nlayer_left): z_top, vp, vs, rho */
    float* fk_right;
    float* c;                   /* c(1:3, NZ, NX) = rho, lambda, mu with rho = (vp + 980) / 2.76 */
} fdfk_input;

int fdfk_input_read(const char* inpath, const char* inparfile, int write_model_copies, fdfk_input* in);
void fdfk_input_free(fdfk_input* in);

/* compute_backazimuth_grids (src/coord_transform.f90) minus the profile azimuth
 * (src/FDFK2D.f90:387): back-azimuths (rad) at profile coordinates coordx[n]. */
int fdfk_backazimuths(double lat_org, double lon_org, double az_org, double evla, double evlo, int n,
                      const float* coordx, double* bazs);

/* check_stability (src/Submain.f90:118-164): the largest stable dt for c. */
int fdfk_stable_dt(int norder, int nx, int nz, int npml, float dx, float dz, const float* c, double* dt_stable);

/* An SU file of ntr traces of ns samples (data trace-major, sample fastest),
 * header words 58 and 59 (1-based, int16) set as the reference sets them. */
int fdfk_write_su(const char* path, int ntr, int ns, const float* data, int head58, int head59);

/*
 * Program FDFK2D (src/FDFK2D.f90) on the GPU: read the input folder, check
 * stability, compute the back-azimuths of the grid, the FK background on the
 * GPU, the time loop with receiver sampling (and snapshots into
 * <outpath>/snapshots/ when the FD model asks for them), project the radial
 * component and write <outpath>/<fsis>x.su and <fsis>z.su ("seis" when fsis
 * is NULL or empty).  Where the reference asks on stdin whether to continue
 * (profile more than 30 degrees off the back-azimuth) this prints a warning
 * and continues.
 */
int fdfk_run(const char* inpath, const char* inparfile, const char* outpath, const char* fsis, int write_model_copies);

/*
 * Batches: many solves advanced together (events of one model, or models of
 * different sizes), each solve the time loop of simulate_wavefield
 * (src/FDFK2D.f90:465-532) on its own session.  No counterpart in the
 * reference, which runs one solve per process.
 *
 * All members share `norder`.  A step of the batch is three kernel launches
 * whatever the number of members (a bookkeeping kernel, the fast path and the
 * tiled kernel over every member's cells); chunks of `graph chunk` steps are
 * captured into a CUDA graph and replayed while the membership is unchanged.
 * A member stops at its own last time index nt.  While a session is a member,
 * calls that change it (advance, upload_*, set_receivers, fk_background) are
 * refused with FDFK_ESTATE; downloads and fdfk_session_synchronize first wait
 * for the batch.  Sessions must have their background for every remaining
 * time index when added.
 */
typedef struct fdfk_batch fdfk_batch;
int fdfk_batch_create(int norder, fdfk_batch** out);
int fdfk_batch_add(fdfk_batch* b, fdfk_session* s);
int fdfk_batch_remove(fdfk_batch* b, fdfk_session* s);
/* Steps per captured graph (default 32; 0 launches step by step). */
int fdfk_batch_set_graph_chunk(fdfk_batch* b, int steps);
/* Launch shapes for every member while in this batch: fast-path segment columns (8..1024; 0 plans
 * them for the batch, about two waves of resident warps) and absorbing-layer tile length (8..64;
 * 0 keeps each member's own).  Results do not depend on either. */
int fdfk_batch_set_tuning(fdfk_batch* b, int seg_len, int pml_run);
/* Advance every member by nsteps (a member past its nt does nothing). Asynchronous. */
int fdfk_batch_advance(fdfk_batch* b, int nsteps);
/* Wait for the batch and bring the members' step counters up to date. */
int fdfk_batch_synchronize(fdfk_batch* b);
/* Members that have not yet passed their last time index (synchronizes). */
int fdfk_batch_live(fdfk_batch* b);
int fdfk_batch_size(const fdfk_batch* b);
/* Releases the batch; its members become ordinary sessions again. */
void fdfk_batch_destroy(fdfk_batch* b);

/*
 * The whole time loop of simulate_wavefield (src/FDFK2D.f90:465-532) in one
 * call: host material and background in, host seismograms out, state zeroed
 * at the start as in src/FDFK2D.f90:280-300.  seisx/seisz are (nsis+1) x nrcv.
 */
int fdfk_simulate(const fdfk_params* p, const float* c, const float* const strips[12], int nrcv, const float* rx,
                  const float* rz, float x0, float z0, int nstp, int nsis, float* seisx, float* seisz);

/*
 * FK background wavefield (replaces lib_gnu/libFK3D.so's
 * comput_background_wavefield_, called at src/FDFK2D.f90:429-431).
 * Scalars of that call, same meaning and precision.
 */
typedef struct fdfk_fk_params {
    int nx, nz, npml;
    int izt;          /* 1 (free surface on top) is the implemented mode */
    int nbd, nt;
    int src_type;     /* reference logical: nonzero = incident P, 0 = incident SV */
    float x0, z0, dx, dz;
    double dt;
    float ds, f0;     /* source scale and Ricker centre frequency */
    double rayp;      /* ray parameter, s/m (the caller clamps |rayp| >= 1e-9) */
} fdfk_fk_params;

/*
 * Computes the 12 background strips on the GPU (FP64 propagators, spectra
 * and transforms; float32 strips) into host arrays in the reference layout.
 * bazs: back-azimuths (rad) of columns 1-npml..nx+npml, profile frame
 * (src/FDFK2D.f90:385-387).  fk_left / fk_right: (4, nlayer) column-major
 * z_top, vp, vs, rho per layer, the last layer the half-space.
 */
int fdfk_fk_background(const fdfk_fk_params* p, const double* bazs, int nlayer_left, const float* fk_left,
                       int nlayer_right, const float* fk_right, float* const strips[12]);

/*
 * Same computation written straight into the session's device-resident
 * strips (all nt+1 time samples), with no host copy of the strips.  The FK
 * geometry (nx, nz, npml, nbd, nt) must match the session's.
 */
int fdfk_session_fk_background(fdfk_session* s, const fdfk_fk_params* p, const double* bazs, int nlayer_left,
                               const float* fk_left, int nlayer_right, const float* fk_right);

/*
 * Serving: solve requests (a model, an incident plane wave, receivers) are
 * queued, admitted in arrival order while their device memory fits the
 * budget (fdfk_session_device_bytes: material, wavefield, absorbing-layer
 * state, the FK background of every time step, seismograms), joined to one
 * running batch and retired into the caller's buffers when done.  No
 * counterpart in the reference.  Each fdfk_server_pump call retires finished
 * solves (waiting for the chunk launched by the previous pump), admits what
 * fits, and launches the next chunk of steps asynchronously; requests that
 * arrive between pumps join the running batch at the next pump.  Every
 * pointer of a request must stay valid until its state is DONE or FAILED.
 * The FK background of an admitted request is computed on the GPU.
 */
#define FDFK_REQ_QUEUED 0
#define FDFK_REQ_RUNNING 1
#define FDFK_REQ_DONE 2
#define FDFK_REQ_FAILED 3

typedef struct fdfk_solve_request {
    fdfk_params p;                 /* grid, stencil, PML; nt = last time index */
    const float* c;                /* c(1:3, NZ, NX) = rho, lambda, mu */
    fdfk_fk_params fk;             /* FK background (geometry as p) */
    const double* bazs;            /* nx + 2 npml back-azimuths (rad) */
    int nlayer_left;
    const float* fk_left;          /* (4, nlayer_left) */
    int nlayer_right;
    const float* fk_right;         /* (4, nlayer_right) */
    int nrcv;                      /* receivers, as fdfk_session_set_receivers */
    const float* rx;
    const float* rz;
    float x0, z0;
    int nstp, nsis;
    float* seisx;                  /* outputs (nsis+1) x nrcv, written when the solve is done */
    float* seisz;
} fdfk_solve_request;

typedef struct fdfk_server_stats {
    int queued, running;
    long long completed, failed;
    long long bytes_in_use, budget;
} fdfk_server_stats;

typedef struct fdfk_server fdfk_server;

/* Device bytes one session of these parameters holds (nrcv receivers, nsis+1 samples). */
long long fdfk_session_device_bytes(const fdfk_params* p, int nrcv, int nsis);
int fdfk_server_create(int norder, long long hbm_budget_bytes, int chunk_steps, fdfk_server** out);
int fdfk_server_submit(fdfk_server* s, const fdfk_solve_request* r, long long* id);
/* Retire, admit, launch one chunk; *in_flight = queued + running requests afterwards. */
int fdfk_server_pump(fdfk_server* s, int* in_flight);
/* State (FDFK_REQ_*) and host steady-clock times (s) of submission, admission and completion. */
int fdfk_server_request(fdfk_server* s, long long id, int* state, double* t_submit, double* t_admit, double* t_done);
int fdfk_server_get_stats(const fdfk_server* s, fdfk_server_stats* st);
void fdfk_server_destroy(fdfk_server* s);

/*
 * Drop-in for lib_gnu/libFK3D.so's comput_background_wavefield_ (32
 * arguments, gfortran ABI, by reference; call at src/FDFK2D.f90:429-431).
 * Prints a message and aborts on failure, as a Fortran `stop` would.
 */
void comput_background_wavefield_(const int* nx, const int* nz, const int* npml, const int* izt, const int* nbd,
                                  const int* nt, const int* nlayer_left, const int* nlayer_right,
                                  const int* src_type, const float* x0, const float* z0, const float* dx,
                                  const float* dz, const double* dt, const float* ds, const float* f0,
                                  const double* rayp, const double* bazs, const float* fk_left,
                                  const float* fk_right, float* uxl_reg, float* uzl_reg, float* uxr_reg,
                                  float* uzr_reg, float* uxb_reg, float* uzb_reg, float* uxl_pml, float* uzl_pml,
                                  float* uxr_pml, float* uzr_pml, float* uxb_pml, float* uzb_pml);

/*
 * One time step with updatedispl_'s meaning (same arrays, same in-place
 * update of ux, uz, bp, bu; strips hold time samples 0..nt and sample `it`
 * is used) that allocates nothing: no counterpart in the reference.  Every
 * device buffer of the call is carved from one file-scope static device array
 * of fdfk_step_noalloc_capacity() floats (16 Mi floats, 64 MiB); a geometry
 * that needs more (fdfk_step_noalloc_need) is rejected with FDFK_EINVAL
 * before any device work.  The call runs on `stream` (NULL: the default
 * stream) and returns after that stream has drained.
 * Races: the scratch is shared by every caller in the process on a device;
 * calls that overlap in time (two host threads, or two streams) corrupt each
 * other - serialise them.  The first call on a device resolves the scratch
 * address (cudaGetSymbolAddress) and the FD coefficient tables go to constant
 * memory once per device; a failed CUDA call drops the cached address, so after
 * a device reset the first call may fail once and the next resolves it again.
 * No call may be made on a stream that is being captured, nor while any
 * global-mode stream capture is in progress: each call does pageable copies
 * and waits for its stream.
 */
int fdfk_step_noalloc(const fdfk_params* p, int it, const float* const strips[12], const float* c, float* ux,
                      float* uz, float* const bp[12], float* const bu[24], void* stream);
long long fdfk_step_noalloc_capacity(void);
long long fdfk_step_noalloc_need(const fdfk_params* p);

/*
 * Drop-in for the shipped libHybrid.so + libPML.so entry point
 * `updatedispl_` (68 arguments, gfortran ABI, everything by reference),
 * called from src/FDFK2D.f90:516-522.  Each call uploads the state, runs one
 * fused step on the GPU and writes the state back into the caller's arrays.
 * A mode this build does not implement prints a message and aborts, as the
 * reference's `stop` would.
 */
void updatedispl_(const int* norder, const int* nx, const int* nz, const int* npml, const int* izt,
                  const int* is_PML_top, const int* npower, const int* nbd, const int* it, const int* nt,
                  const float* dx, const float* dz, const double* dt, const float* vpml, const double* R0,
                  const float* uxl_reg, const float* uzl_reg, const float* uxr_reg, const float* uzr_reg,
                  const float* uxb_reg, const float* uzb_reg, const float* uxl_pml, const float* uzl_pml,
                  const float* uxr_pml, const float* uzr_pml, const float* uxb_pml, const float* uzb_pml,
                  const float* c, const double* coef0, const double* coef1, float* ux, float* uz,
                  float* bpxlx, float* bpzlx, float* bpxrx, float* bpzrx, float* bpxtx, float* bpxtz, float* bpztx,
                  float* bpztz, float* bpxbx, float* bpxbz, float* bpzbx, float* bpzbz,
                  float* bux1l, float* bux2l, float* bux3l, float* buz1l, float* buz2l, float* buz3l,
                  float* bux1r, float* bux2r, float* bux3r, float* buz1r, float* buz2r, float* buz3r,
                  float* bux1b, float* bux2b, float* bux3b, float* buz1b, float* buz2b, float* buz3b,
                  float* bux1t, float* bux2t, float* bux3t, float* buz1t, float* buz2t, float* buz3t);

#ifdef __cplusplus
}
#endif
#endif
