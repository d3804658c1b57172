/*
 * wave.h — C ABI of the GB300-native forward solver for the WAVE-Simulation
 * time-stepping hot path (ForwardSolver::run and everything it calls).
 *
 * Every entry point returns an int status (WAVE_OK on success). No C++
 * exception and no pointer owned by the library ever crosses this boundary.
 * A handle is bound to one CUDA device and one CUDA stream; handles are not
 * thread-safe, use one handle per host thread (the reference calls
 * ForwardSolver::run from one thread per MPI rank, Simulation.cpp:452).
 *
 * Axis convention (same as the reference, Coordinates.cpp:615-644):
 *   x = horizontal inline (fastest), z = horizontal crossline, y = depth
 *   (slowest); linear index idx = x + z*NX + y*NX*NZ. 2-D runs use NZ = 1.
 */
#ifndef WAVE_GB300_H
#define WAVE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (replace COMMON_THROWEXCEPTION / SCAI_ASSERT_ERROR) ---- */
#define WAVE_OK 0
#define WAVE_ERR_ARG 1          /* invalid argument, size mismatch, null handle   */
#define WAVE_ERR_CUDA 2         /* a CUDA runtime call failed                      */
#define WAVE_ERR_NONFINITE 3    /* NaN/Inf found in the wavefield or seismogram    */
#define WAVE_ERR_TIMEOUT 4      /* a bounded device-side wait ran out              */
#define WAVE_ERR_UNSUPPORTED 5  /* dimension/equation combination not available   */
#define WAVE_ERR_STATE 6        /* call out of order (e.g. step before set_model)  */
#define WAVE_ERR_IO 7           /* file could not be read or parsed               */

/* ---- equation types: the ForwardSolver factory keys
 *      (ForwardSolver/ForwardSolverFactory.cpp:4-67) ---- */
#define WAVE_EQ_ACOUSTIC 0
#define WAVE_EQ_ELASTIC 1
#define WAVE_EQ_VISCOELASTIC 2
#define WAVE_EQ_SH 3
#define WAVE_EQ_VISCOSH 4
#define WAVE_EQ_TMEM 5
#define WAVE_EQ_EMEM 6
#define WAVE_EQ_VISCOTMEM 7
#define WAVE_EQ_VISCOEMEM 8

/* ---- seismogram / source component types (Acquisition/Acquisition.hpp:17-44)
 *      seismic: 1=P 2=VX 3=VY 4=VZ ; EM: 1=EZ 2=EX 3=EY 4=HZ ---- */
#define WAVE_TYPE_P 1
#define WAVE_TYPE_VX 2
#define WAVE_TYPE_VY 3
#define WAVE_TYPE_VZ 4
#define WAVE_TYPE_EZ 1
#define WAVE_TYPE_EX 2
#define WAVE_TYPE_EY 3
#define WAVE_TYPE_HZ 4

/* ---- memory flags for pointer arguments ---- */
#define WAVE_MEM_HOST 0
#define WAVE_MEM_DEVICE 1

/*
 * Solver configuration: the hot-path subset of the reference's
 * Configuration keys (Configuration/Configuration.cpp:45-100, keys as read by
 * Simulation.cpp, Derivatives.cpp:12-55 and ForwardSolver.cpp:34-54).
 */
#define WAVE_MAX_GRID_LAYERS 16

typedef struct wave_config {
    int dimension;              /* "dimension": 2 or 3                               */
    int equation;               /* "equationType": WAVE_EQ_*                         */
    int64_t NX, NY, NZ;         /* "NX","NY","NZ" (NY = depth; NZ = 1 in 2-D)       */
    double DH;                  /* "DH"  grid spacing [m]                            */
    double DT;                  /* "DT"  time step [s]                               */
    double T;                   /* "T"   record length [s]; NT = int(T/DT + 0.5)    */
    int spatialFDorder;         /* "spatialFDorder": 2,4,6,8,10,12                   */
    int FreeSurface;            /* "FreeSurface": 0 none, 1 mirror/image method      */
    int DampingBoundary;        /* "DampingBoundary": 0 none, 1 ABS, 2 CPML          */
    int BoundaryWidth;          /* "BoundaryWidth" [grid points]                     */
    double DampingCoeff;        /* "DampingCoeff" [%] (ABS)                          */
    double NPower;              /* "NPower" (CPML)                                   */
    double CenterFrequencyCPML; /* "CenterFrequencyCPML" [Hz] (CPML, visco ref. f)   */
    double VMaxCPML;            /* "VMaxCPML" [m/s] (CPML)                           */
    int numRelaxationMechanisms;       /* "numRelaxationMechanisms" (0..4)           */
    double relaxationFrequency[4];     /* "relaxationFrequency", "...2", "...3", "...4" */
    int useStencilMatrix;       /* "useStencilMatrix": 0 = sparse (CSR) operators,
                                   1 = stencil operators (always zero-padded)      */
    int edgeOrderReduction;     /* sparse operators only. 1 = reduce the FD order at
                                   the grid edges until the stencil fits, as the
                                   current Derivatives.cpp:166-179, 743-756 does;
                                   0 = drop neighbours outside the grid (zero
                                   padding), the rule the reference's CI golden
                                   seismograms (par/ci, seismogram.<case>.ref.<c>.mtx)
                                   were made with.
                                   Config key "edgeOrderReduction" (default 1).   */
    /* Variable (discontinuous) grid, Acquisition/Coordinates.cpp:35-245 and
     * Derivatives.cpp:852-1656. Acoustic equations (2-D and 3-D, free
     * surface allowed) and elastic (2-D and 3-D, FD2Delastic / FD3Delastic
     * ::run with the staggered-x / -z y-derivatives, FreeSurface 0 or 1);
     * CPML, ABS or no damping boundary; no adjoint. The grid's index space replaces NX*NY*NZ
     * everywhere (model arrays, source/receiver indices, wavefields): see
     * wave_grid_*. */
    int useVariableGrid;        /* "useVariableGrid": layers of spacing DH*dhFactor   */
    int useVariableFDoperators; /* "useVariableFDoperators": FD order per layer      */
    int gridLayers;             /* rows of "gridConfigurationFilename" (1..16)       */
    int gridInterface[WAVE_MAX_GRID_LAYERS]; /* column 0: first depth index of each
                                   layer (the first is 0)                          */
    int gridDHFactor[WAVE_MAX_GRID_LAYERS];  /* column 1: spacing factor, 3^n        */
    int gridFDOrder[WAVE_MAX_GRID_LAYERS];   /* column 2: FD order of the layer      */
} wave_config;

typedef struct wave_handle wave_handle;

/* Number of time samples the reference uses: int(T/DT + 0.5) evaluated in
 * single precision (Common/Common.hpp:240-243, Sources.cpp:26). */
int wave_config_nt(const wave_config* cfg, int* nt);

/* Parse a reference parameter file (KEY=VALUE, '#' comments, keys
 * case-insensitive) into *cfg. Replaces Configuration::Configuration(file)
 * + the get<T>() calls of the hot path (Configuration/Configuration.cpp:45-100,
 * Configuration.hpp:95-143). Missing mandatory keys -> WAVE_ERR_ARG. */
int wave_config_from_file(const char* path, wave_config* cfg);

/* Grid index space of a configuration: NX*NY*NZ points in the reference
 * order x + z*NX + y*NX*NZ, or the variable grid's layered points
 * (Coordinates::getNGridpoints, Coordinates.cpp:340-346). */
int wave_grid_num_points(const wave_config* cfg, int64_t* n);
/* Coordinates::coordinate2index (Coordinates.cpp:668-698): 1-D index of the
 * fine-grid coordinate (x, y, z); on a coarse layer the coordinate is rounded
 * down to the layer's points. WAVE_ERR_ARG outside the grid. */
int wave_grid_index(const wave_config* cfg, int64_t x, int64_t y, int64_t z, int64_t* idx);
/* Coordinates::index2coordinate (Coordinates.cpp:603-650) for every index:
 * x, y, z receive n = wave_grid_num_points values each. Also returns the
 * extents the variable grid reduced NX, NY, NZ to (NULL to skip). */
int wave_grid_coordinates(const wave_config* cfg, int64_t* x, int64_t* y, int64_t* z, int64_t n, int64_t* extents3);
/* The assembled sparse operator `op` of a variable-grid configuration
 * (host only, no GPU): 0 Dxf, 1 Dyf (DyfFreeSurface with FreeSurface=1),
 * 2 Dzf, 3 Dxb, 4 Dyb, 5 Dzb, DT folded in (Derivatives.cpp:129-1245,
 * FDTD2D.cpp:193-229), the interface interpolation 6 Full, 7 StaggeredX,
 * 8 StaggeredZ (Derivatives.cpp:1252-1546; rows off the interfaces are the
 * identity), the elastic staggered y-derivatives 9 DyfStaggeredX,
 * 10 DybStaggeredX (Derivatives.cpp:852-1011), 11 DyfStaggeredZ,
 * 12 DybStaggeredZ (Derivatives.cpp:1012-1168, 3-D; with FreeSurface=1,
 * 10 and 12 are DybStaggeredX / ZFreeSurface, :533-704), or 13 the interface
 * interpolation StaggeredXZ (Derivatives.cpp:1568-1661, 3-D). Returned as an
 * ELL block: *width entries per row, entry k of row i at k*N + i, unused
 * entries with weight 0. With cols == NULL only *width is set; otherwise
 * capacity must be at least width * N. */
int wave_grid_operator(const wave_config* cfg, int op, int* width, int32_t* cols, float* vals, int64_t capacity);

/* ForwardSolver::Factory<float>::Create(dimension, type)
 * (ForwardSolver/ForwardSolverFactory.cpp:4-67) followed by initForwardSolver
 * (ForwardSolver.hpp:52, e.g. ForwardSolver3Delastic.cpp:20-48): validates the
 * combination, allocates device state (wavefields, memory variables, CPML psi
 * slabs) on the current CUDA device and builds the boundary tables. */
int wave_solver_create(const wave_config* cfg, wave_handle** out);
int wave_solver_destroy(wave_handle* h);

/* Modelparameter init + Modelparameter::prepareForModelling (e.g.
 * Elastic.cpp:28-45, Viscoelastic.cpp:650-715, ModelparameterSeismic.cpp:
 * 131-136, 421-432, Modelparameter.cpp:336-651) + the solver's
 * prepareForModelling (ForwardSolver.hpp:42, e.g. ForwardSolver3Dviscoelastic.cpp:103-118,
 * FreeSurfaceElastic.cpp:11-47). Arrays have n = wave_grid_num_points entries
 * (NX*NY*NZ on a regular grid) in the reference index order; unused parameters may be NULL (vs for acoustic,
 * vp for sh, taup/taus unless visco). mem = WAVE_MEM_HOST or WAVE_MEM_DEVICE. */
int wave_set_model(wave_handle* h, const float* rho, const float* vp, const float* vs,
                   const float* taup, const float* taus, size_t n, int mem);

/* EM counterpart (ModelparameterEM/TMEM.cpp:145-170, 230-241; ForwardSolverEM.cpp:14-117):
 * eps_r relative permittivity, sigma conductivity [S/m], mu_r relative
 * permeability; tau_eps / tau_sigma for the visco-EM equations (else NULL). */
int wave_set_model_em(wave_handle* h, const float* eps_r, const float* sigma, const float* mu_r,
                      const float* tau_eps, const float* tau_sigma, size_t n, int mem);

/* Source coupling (SourceReceiverImpl.cpp:29-37): n sources at 1-D grid
 * indices idx, component types type[] (WAVE_TYPE_*), signals n x NT row-major
 * (source i's trace is signals[i*NT .. i*NT+NT-1]); the raw sample of column t
 * is added at step t. */
int wave_set_sources(wave_handle* h, int n, const int64_t* idx, const int* type,
                     const float* signals, int mem);

/* Receiver gather (SourceReceiverImpl.cpp:12-19, FDTD*elastic.cpp pressure
 * averages): n receivers at 1-D indices idx with component types type[]. */
int wave_set_receivers(wave_handle* h, int n, const int64_t* idx, const int* type);

/* ForwardSolver::run(receiver, sources, model, wavefield, derivatives, t) for
 * every t in [t_begin, t_end) (ForwardSolver.hpp:38, caller Simulation.cpp:444-476).
 * A multi-step call runs as one captured CUDA graph; a one-step call keeps the
 * reference's run(t) granularity. Asynchronous on the handle's stream. */
int wave_solver_step(wave_handle* h, int t_begin, int t_end);

/* Wavefields::resetWavefields + ForwardSolver::resetCPML (ForwardSolver.hpp:40,
 * Simulation.cpp:432, :514): zero all wavefields, memory variables, psi and
 * the seismogram buffer. */
int wave_solver_reset(wave_handle* h);

/* Receiver seismograms, n_receivers x NT row-major, trace order = the order
 * given to wave_set_receivers. Synchronises the handle's stream. */
int wave_get_seismograms(wave_handle* h, float* out, size_t count, int mem);

/* NaN/Inf check of the wavefields and seismograms (Simulation.cpp:519,
 * WavefieldsSeismic.cpp:12-40) done on the device over every point:
 * returns WAVE_OK or WAVE_ERR_NONFINITE. */
int wave_check_finite(wave_handle* h);

/* Full solver state (wavefields, memory variables, CPML psi slabs) as one
 * blob, for checkpoint / resume. The reference has no counterpart (it only
 * writes snapshots, Simulation.cpp:468-475). */
int wave_get_state_size(wave_handle* h, size_t* bytes);
int wave_get_state(wave_handle* h, void* out, size_t bytes, int mem);
int wave_set_state(wave_handle* h, const void* in, size_t bytes, int mem);

/* Query helpers. */
int wave_get_nt(wave_handle* h, int* nt);
/* Device memory the handle holds (wavefields, memory variables, materials,
 * CPML slabs, operator tables, acquisition and seismogram buffers), in bytes.
 * Replaces ForwardSolver::estimateMemory plus the wavefield/model estimates
 * Simulation.cpp:169-174 prints (ForwardSolver.hpp:46), measured instead of
 * estimated. */
int wave_device_bytes(wave_handle* h, int64_t* bytes);
int wave_get_num_receivers(wave_handle* h, int* n);
/* Device pointer to the CUDA stream the handle launches on (cudaStream_t). */
int wave_get_stream(wave_handle* h, void** stream);
/* Number of kernels launched by this handle since creation (memory copies
 * and memsets are not counted). */
int wave_get_launch_count(wave_handle* h, long long* count);
/* Average duration [ms] of the most recent timed step kernels, measured with
 * CUDA events on the handle's stream when timing is on (see wave_set_timing). */
int wave_set_timing(wave_handle* h, int on);
int wave_get_kernel_times(wave_handle* h, double* velocity_ms, double* stress_ms, long long* samples);

/* Harmonic S-wave-modulus average with the reference's vacuum rules
 * (ModelparameterSeismic::calcAveragedSWaveModulus, ModelparameterSeismic.cpp:421-432):
 * moduli below 1 are raised to 1, their inverses are averaged over the 4 points
 * of a grid plane with the edge fallbacks of Modelparameter.cpp:448-527
 * (mode 0 = XY, 1 = XZ, 2 = YZ) or over 2 points along an axis (mode 3 = x,
 * 4 = y; the SH models, SH.cpp:429-430), and averages below 4 become 0.
 * mu and out hold NX*NY*NZ values in the reference index order, both on the
 * host or both on the current CUDA device (mem). Synchronous; no handle. */
int wave_average_shear_modulus(const float* mu, float* out, int64_t NX, int64_t NY, int64_t NZ, int mode, int mem);

/* The same average without any device allocation. No counterpart in the
 * reference (its LAMA matrices own their storage).
 * For callers that must not allocate device memory: an FWI loop that updates
 * the model between iterations while the wavefields, checkpoints and
 * gradients fill the device (a cudaMalloc there can fail), and code that
 * cannot accept the device-wide synchronisation cudaMalloc/cudaFree imply.
 * mu and out are device pointers on the current device (out may equal mu);
 * the work is queued on `stream` (a cudaStream_t, NULL = legacy default
 * stream) and the call returns without waiting.
 * Limit: NX*NY*NZ <= 4194304 (2^22) points; the inverse moduli go to a fixed
 * 16 MiB scratch array in device global memory. Larger models return
 * WAVE_ERR_ARG: use wave_average_shear_modulus.
 * The first call on each device does a one-time set-up (it looks up the
 * scratch array's address with that device current); make that first call
 * before any stream capture. Nothing has to start at zero: every scratch
 * value that is read was written earlier in the same call. The scratch is
 * shared by all calls on a device, so calls that overlap in time (other
 * streams, other host threads) race on it and must be serialised by the
 * caller. The scratch address is looked up once per device and kept for the
 * life of the process: do not call this entry point on a device after a
 * cudaDeviceReset. The C ABI cannot check the length of mu and out: both
 * must hold NX*NY*NZ floats. A CUDA error left pending by earlier work is
 * reported as WAVE_ERR_CUDA before anything is launched (and not cleared). */
int wave_average_shear_modulus_noalloc(const float* mu, float* out, int64_t NX, int64_t NY, int64_t NZ, int mode, void* stream);

/* Kernel path: 0 = automatic, 1 = generic kernels only (and the separate
 * source/receiver kernel: by default, acoustic grids of at most 2^20 points
 * with pressure sources and no ABS add the sources and record the receivers
 * inside the pressure kernel, one launch less per step), 2 = the one-point
 * streaming TMA kernels wherever they apply (3-D elastic grids with
 * NX % 4 == 0 whose 32x8 column tiles meet at most one CPML slab per axis),
 * 3 = the two-points-per-thread streaming kernels wherever they apply (64x8
 * tiles, even x CPML slab width). The automatic path times the generic
 * kernel and the streaming kernel that applies (the two-point one where it
 * applies) of each pass when the model is set on an unstepped state and keeps
 * the faster per pass. wave_get_kernel_path reports which passes run a
 * streaming kernel (bit 0 velocity pass, bit 1 stress pass) and which of those
 * run the two-point kernels (bit 2 velocity, bit 3 stress). The reference has
 * no counterpart (LAMA picks its own SpMV kernels). */
int wave_set_kernel_path(wave_handle* h, int path);
int wave_get_kernel_path(wave_handle* h, int* streaming_active);

/* Programmatic dependent launch of the one-thread-per-point kernels, the ABS
 * frame and the source/receiver kernel (on = 1, the default): each such
 * launch may be scheduled before its predecessor in the stream has finished
 * and waits for it inside the kernel, so the launch latency between the
 * 3-4 kernels of a step is hidden on small grids. Results do not depend on
 * this switch. The reference has no counterpart. */
int wave_set_dependent_launch(wave_handle* h, int on);

/* Wavefield decomposition after every step (config key decomposeWavefieldType,
 * Simulation.cpp:316, 450-461; FD2Dacoustic::decompose, Wavefields2Dacoustic.cpp:
 * 119-300; FD2Dtmem::decompose, Wavefields2Dtmem.cpp:109-160): type 1 splits
 * P, VX, VY (TMz: EZ) into up- and down-going parts, type 2 into left- and
 * right-going parts, by the sign of S2 * max|S1|/max|S2| + S1 with
 * S1 = -P*VY (resp. -P*VX; TMz: EZ*HX, resp. -EZ*HY) and
 * S2 = -(Dyf F)(dF/dt) (resp. Dxf); 0 turns it off. 2-D acoustic and 2-D TMz
 * on a regular grid (the reference's other decompositions are empty). The
 * parts are read with wave_get_field under the reference's file-name tokens
 * "P.up", "P.down", "VX.up", ..., "P.left", ..., "EZ.up", "EZ.left", .... The reference's Dyf is empty for
 * acoustic modelling with a free surface (FDTD2D.cpp:258-262), which makes
 * its type-1 parts undefined there; this library applies Dyf regardless. */
int wave_set_decomposition(wave_handle* h, int type);

/* Source encoding (config keys useSourceEncode, NumShotDomains;
 * Sources::calcSourceSettingsEncode, Acquisition/Sources.cpp:569-660, for
 * time-domain modelling): the n shots (one source row each; shot_no and amp
 * as read from the source file) are regrouped into num_domains super-shots.
 * mode 1: the first num_domains shots go to super-shots 0.. in order, the
 * others to random super-shots that are not yet full (at most
 * ceil(n / num_domains) shots each), then each amplitude's sign is flipped at
 * random; mode 2: shot i to super-shot i % num_domains; mode 3: contiguous
 * runs of ceil(n / num_domains) shots. shot_no_out[i] = num_domains*10^4 + 1 +
 * super-shot; amp_out the (signed) amplitudes. Random numbers are the C
 * library's rand() after srand(seed) (the reference seeds with time(0)).
 * Host only. The receiver side (Receivers.cpp:354-573) is wave_encode_traces. */
int wave_encode_sources(int mode, int num_domains, unsigned int seed, int n, const int* shot_no, const float* amp,
                        int* shot_no_out, float* amp_out);
/* The frequency list of the frequency-domain encoding (gradientDomain != 0,
 * Sources.cpp:587-611): df = 1 / (nFFT DT) with nFFT the next power of two of
 * NT - 1 (NT = T / DT + 0.5), band indices ceil(fc / df) (fc2 = 0: twice the
 * CPML centre frequency). encoded != 0: every second frequency from an even
 * first index (the list the super-shots draw from); encoded = 0: every
 * frequency of the widened band [ceil(i1 / 2), 2 i2] (the per-shot list of
 * unencoded frequency-domain modelling). Writes min(cap, n) frequencies to
 * freqs (may be null) and n to *nfreq. Host only. */
int wave_encode_frequencies(int encoded, double fc1, double fc2, double T, double DT, double cpml_fc, float* freqs, int cap,
                            int* nfreq);
/* Frequency-domain source encoding: wave_encode_sources' super-shot
 * assignment (the same rand() stream), then each shot of a super-shot draws a
 * distinct random frequency of the encoded list (Sources.cpp:641-660); the
 * reference then models each shot with wavelet shape 9 (sin) at fc_out[i].
 * WAVE_ERR_ARG when the list holds fewer frequencies than shots per
 * super-shot. Host only. */
int wave_encode_sources_frequency(int mode, int num_domains, unsigned int seed, int n, const float* amp, double fc1, double fc2,
                                  double T, double DT, double cpml_fc, int* shot_no_out, float* amp_out, float* fc_out);
/* Receiver-side encoding of seismograms for one receiver component
 * (Receivers::encode / Receivers::decode, Receivers.cpp:354-573): the shots of
 * one super-shot summed into its receiver rows (decode = 0) or split back out
 * (decode = 1). mark: nshots x nrec (receiver r recorded for shot s when
 * nonzero), super_mark: nrec (receiver r is in the super-shot), amp: the
 * shots' encoded amplitudes (a negative one flips the shot's traces), fc:
 * the shots' frequencies (null: no filter; else the single-frequency ideal
 * band-pass of frequency-domain modelling, Filter.cpp:239-342, with DT).
 * Multi-offset data (common_offset = 0): shot_data[s] holds the rows of the
 * shot's marked receivers among the super-shot's, in receiver order;
 * super_data one row per super-shot receiver; the filter is the block form
 * (2 / nFFT, then divided by the block's largest magnitude). Common-offset
 * data (common_offset = 1, nshots == nrec): one trace per shot, super row k
 * the k-th shot whose receiver is in the super-shot, added (or received) only
 * where the shot's own receiver is marked for it (elsewhere the decoded trace
 * is zero), the single-trace filter (1 / NT). Rows are nt samples; shot_data
 * is a host array of nshots pointers, all data in `mem`. */
int wave_encode_traces(int decode, int nshots, int nrec, int64_t nt, const int* mark, const int* super_mark, const float* amp,
                       const float* fc, double DT, int common_offset, float* const* shot_data, float* super_data, int mem);

/* ---- seismogram output path and file formats ---- */
/* Resampling of ntr traces (row-major ntr x nt, sample interval dt) to
 * seismo_dt by linear interpolation (Common::calcResampleMat,
 * Common.hpp:202-230, applied as data * resampleMat in Seismogram::write,
 * Seismogram.cpp:109); seismo_dt = 0 keeps dt. *nt_out receives
 * floor((nt-1) / (seismo_dt/dt)) + 1; with out == NULL only *nt_out is set.
 * in/out on the host or the current device (mem). */
int wave_resample_traces(const float* in, int64_t ntr, int64_t nt, double dt, double seismo_dt, float* out, int64_t* nt_out, int mem);
/* Seismogram::normalizeTrace (Seismogram.cpp:215-275) in place: mode 0 none,
 * 1 each trace divided by its max |value|, 2 by its l2 norm (a zero norm
 * divides by 1), 4 l2 norm then division by the envelope plus 1e-3 of its
 * maximum. Mode 3 (AGC) needs dt and the AGC frequency: wave_agc_normalize_traces. */
int wave_normalize_traces(float* data, int64_t ntr, int64_t nt, int mode, int mem);
/* AGC normalisation, normalizeTraces = 3 (Seismogram::calcInverseAGC,
 * Seismogram.cpp:323-387, then normalizeTrace(3), :235-237), in place: the
 * inverse AGC of the l2-normalised traces over a window of round(1/(f_agc dt))
 * samples on each side (at most nt/2; the reference passes
 * CenterFrequencyCPML as f_agc), then data = l2-normalised data x inverse AGC.
 * inverse_agc (ntr x nt, may be NULL) receives the inverse AGC, which the
 * reference writes as <seismogram>.<component>.inverseAGC.mtx. */
int wave_agc_normalize_traces(float* data, int64_t ntr, int64_t nt, double dt, double f_agc, float* inverse_agc, int mem);
/* MatrixMarket files (IO::readVector/writeMatrix with fileFormat 1, IO.hpp:21-145):
 * read "array" or "coordinate" real files into a row-major rows x cols buffer
 * (out == NULL: dimensions only); write a row-major matrix in array format. */
int wave_read_mtx(const char* path, float* out, int64_t capacity, int64_t* rows, int64_t* cols);
int wave_write_mtx(const char* path, const float* data, int64_t rows, int64_t cols);
/* SeismicUnix traces with the trace headers of SUIO::writeSU (SUIO.hpp:156-262):
 * ntr x ns row-major samples, receiver and source grid indices, grid and DH. */
int wave_write_su(const char* path, const float* data, int64_t ntr, int64_t ns, double dt, const int64_t* rec_idx, int64_t src_idx,
                  int64_t NX, int64_t NY, int64_t NZ, double DH);

/* Diagnostic of the device-side failure path: runs the streaming kernels'
 * bounded mbarrier wait on a barrier that never completes; *status receives
 * WAVE_ERR_TIMEOUT when the wait gave up as designed (the context stays
 * usable). No counterpart in the reference. */
int wave_selftest_bounded_wait(int* status);

/* ---- snapshots and trace attributes ---- */
/* One wavefield of the handle ("VX", "VY", "VZ", "P", "Sxx", ..., "Syz", "HX",
 * "HY", "HZ", "EX", "EY", "EZ"; case-insensitive) into out (N floats), the
 * data Wavefields::write stores for snapType 1/2 (Wavefields3Delastic.cpp:62-96). */
int wave_get_field(wave_handle* h, const char* name, float* out, int mem);
/* snapType 3 energies of (visco-)elastic wavefields with the solver's
 * operators: 2-D curl = (Dyf vx - Dxf vy) sqrt(mu), div = (Dxb vx + Dyb vy)
 * sqrt(M) (Wavefields2Delastic.cpp:218-250); 3-D curl = sqrt(mu |curl v|^2),
 * div = sqrt(M (div v)^2) (Wavefields3Delastic.cpp:197-240). */
int wave_get_curl_div(wave_handle* h, float* curl, float* div, int mem);
/* Envelope sqrt(x^2 + H(x)^2) of ntr traces in place, H the FFT Hilbert
 * transform on the next power of two of nt-1 samples (Common::calcEnvelope,
 * Common.hpp:272-290, HilbertFFT.cpp). */
int wave_envelope(float* data, int64_t ntr, int64_t nt, int mem);
/* Common::calcInstantaneousPhase (Common.hpp:297-345) in place, phase type 1
 * (atan), 2 (atan2) or 3 (unwrapped); as there, the imaginary part is -data
 * (the Hilbert call of that function is commented out in the reference). */
int wave_instantaneous_phase(float* data, int64_t ntr, int64_t nt, int phase_type, int mem);

/* ---- adjoint gradient (new; the reference's inversion is a separate project) ----
 * Gradient of J = 1/2 sum over receivers and steps of (d - d_obs)^2 by the
 * discrete adjoint of the time step:
 *  - 2-D and 3-D acoustic (FD2Dacoustic::run, ForwardSolver2Dacoustic.cpp:
 *    91-194; FD3Dacoustic::run, ForwardSolver3Dacoustic.cpp:91-233) with CPML,
 *    ABS or no damping boundary and with or without the free surface
 *    (FreeSurface 1 or 2): grad_vp and grad_rho receive dJ/dvp, dJ/drho, grad_vs
 *    is set to zero;
 *  - 2-D and 3-D elastic (FD2Delastic::run, ForwardSolver2Delastic.cpp:117-297;
 *    FD3Delastic::run, ForwardSolver3Delastic.cpp:120-414) with CPML, ABS or
 *    no damping boundary and with or without the free surface (FreeSurface 1 or 2):
 *    grad_vp, grad_vs, grad_rho receive dJ/dvp, dJ/dvs, dJ/drho;
 *  - 2-D and 3-D visco-elastic (FD2Dviscoelastic::run, ForwardSolver2D
 *    viscoelastic.cpp:130-321; FD3Dviscoelastic::run, ForwardSolver3D
 *    viscoelastic.cpp:132-457) with CPML, ABS or no damping boundary and with
 *    or without the free surface (FreeSurface 1 or 2): the same three outputs, the
 *    relaxation times (tau_p, tau_s) held fixed;
 *  - 2-D SH and visco-SH (FD2Dsh::run, ForwardSolver2Dsh.cpp:108-196;
 *    FD2Dviscosh::run, ForwardSolver2Dviscosh.cpp:126-244, tau_s fixed) with
 *    CPML, ABS or no damping boundary and with or without the free surface:
 *    grad_vs and grad_rho receive dJ/dvs, dJ/drho, grad_vp is set to zero;
 *  - 2-D TMz and visco-TMz (FD2Dtmem::run, ForwardSolver2Dtmem.cpp:108-174;
 *    FD2Dviscotmem::run, ForwardSolver2Dviscotmem.cpp:130-205, tau_eps and
 *    tau_sigma fixed) with
 *    Ez sources and receivers, CPML, ABS or no damping boundary: the three
 *    outputs receive dJ/deps_r, dJ/dsigma, dJ/dmu_r (the model's relative
 *    permittivity, conductivity and relative permeability);
 *  - 2-D TEz and visco-TEz (FD2Demem::run, ForwardSolver2Demem.cpp:112-185;
 *    FD2Dviscoemem::run, ForwardSolver2Dviscoemem.cpp:142-228, taus fixed) with
 *    Ex, Ey and Hz sources and receivers, CPML, ABS or no damping boundary:
 *    the same three outputs;
 *  - 3-D EM and visco-EM (FD3Demem::run, ForwardSolver3Demem.cpp:119-237;
 *    FD3Dviscoemem::run, ForwardSolver3Dviscoemem.cpp:161-309, taus fixed)
 *    with CPML, ABS or no damping boundary: the same three outputs;
 * the acoustic and elastic equations also on a variable grid
 * (useVariableGrid / useVariableFDoperators; vargrid.cu). Runs the
 * forward over all NT steps from a zero state (the handle's sources and
 * receivers; seismograms are left as computed), saving the state every
 * `checkpoint_every` steps, then the backward sweep, recomputing each
 * checkpoint segment. d_obs: n_receivers x NT (dobs_mem host or device);
 * grad_*: N floats each (grad_mem). *misfit receives J. */
int wave_adjoint_gradient(wave_handle* h, const float* dobs, int dobs_mem, int checkpoint_every, double* misfit,
                          float* grad_vp, float* grad_vs, float* grad_rho, int grad_mem);

/* ---- batches of shots (the shot parallelism of Simulation.cpp:116-121, 339-369
 *      as one device-wide launch per pass) ---- */
typedef struct wave_batch wave_batch;

/* nshots configurations that share dimension, equation, order, DT, T, boundary
 * type, free surface and relaxation mechanisms; grid sizes may differ. */
int wave_batch_create(const wave_config* cfgs, int nshots, wave_batch** out);
int wave_batch_destroy(wave_batch* b);
/* The per-shot handle, for wave_set_model*, wave_set_sources,
 * wave_set_receivers, wave_get_seismograms and wave_check_finite. Owned by
 * the batch; do not destroy it or step it on its own. */
int wave_batch_shot(wave_batch* b, int shot, wave_handle** h);
/* Steps t in [t_begin, t_end) of every shot: per step one launch per pass
 * over all shots' tiles and one source/receiver launch; multi-step calls
 * replay a captured CUDA graph. Returns after the steps completed. */
int wave_batch_step(wave_batch* b, int t_begin, int t_end);
/* Adjoint gradients of all shots of a batch (wave_adjoint_gradient per shot,
 * every launch covering all shots). dobs[s]: n_receivers(s) x NT; misfits[s]
 * receives shot s's J; with sum_shots = 1 (shots on one grid) the gradients of
 * all shots are summed into grad_*[0], else grad_*[s] receive shot s's. */
int wave_batch_adjoint_gradient(wave_batch* b, const float* const* dobs, int dobs_mem, int checkpoint_every, double* misfits,
                                float* const* grad_vp, float* const* grad_vs, float* const* grad_rho, int grad_mem, int sum_shots);
/* Schedule of the batched launches (no counterpart in the reference, whose
 * shots run one after another, Simulation.cpp:339-369): each launch's blocks
 * walk the (shot, tile) work list with a grid stride. tile_cols (a multiple of
 * 32) x tile_rows (a multiple of 8) points per work-list entry; blocks_per_sm
 * persistent 256-thread blocks per SM (at most the resident count), or 0 for
 * one block per entry. wave_batch_set_schedule fixes it (0, 0 returns to the
 * autotuner); otherwise the first step call of an unstepped batch times every
 * candidate (tile 32 or 64 wide, 8/16/32/64 rows; 0/1/2/4/8 blocks per SM;
 * one untimed and two timed steps each, state reset afterwards) and keeps the
 * fastest, cached for the process per (equation, FD order, log2 of the mean
 * points per shot, log2 of the shot count). wave_batch_get_schedule reports
 * the schedule and where it came from (source: 0 default, 1 timed by this
 * batch, 2 from the cache, 3 set by the caller). Every schedule gives the same
 * results bit for bit: each grid point's update does not depend on the
 * tiling. */
int wave_batch_set_schedule(wave_batch* b, int tile_cols, int tile_rows, int blocks_per_sm);
int wave_batch_get_schedule(wave_batch* b, int* tile_cols, int* tile_rows, int* blocks_per_sm, int* source);
int wave_batch_get_stream(wave_batch* b, void** stream);
int wave_batch_get_launch_count(wave_batch* b, long long* count);
const char* wave_batch_last_error(const wave_batch* b);

/* Text of the last error on this handle (or of the last failed create when
 * h == NULL). Never NULL. */
const char* wave_last_error(const wave_handle* h);

/* Source time functions of the reference (Sources.cpp:157-215 shapes 1..9:
 * 1 Ricker, 2 SinW, 3 SinThree, 4 FGaussian, 5 Spike, 6 IntgSinThree,
 * 7 Ricker_GprMax, 8 Berlage, 9 Sin) evaluated at t = k*DT, k < NT. */
int wave_wavelet(int shape, int nt, double dt, double fc, double amp, double tshift, float* out);

#ifdef __cplusplus
}
#endif
#endif /* WAVE_GB300_H */
