/*
 * wipems_fdtd.h -- C ABI of the GB300 FDTD engine (libwipems_fdtd.so).
 *
 * Three layers, each replacing one piece of the openEMS call chain that the
 * reference runs on the host CPU:
 *
 *   scene     stand-in for the CSXCAD geometry/material database and the
 *             openEMS XML <FDTD> setup (openems.cpp:798-936): rectilinear mesh
 *             lines, priority-ordered boxes of material / metal / lumped
 *             element / excitation / probe, boundary conditions, pulse.
 *   operator  Operator::CalcECOperator and the operator extensions' builds
 *             (FDTD/operator.cpp:973-1084, operator_ext_upml.cpp:365-466,
 *             operator_ext_lorentzmaterial.cpp:117-438,
 *             operator_ext_excitation.cpp:101-285).  Produces the reference's
 *             own per-edge FP32 coefficient arrays (vv/vi/ii/iv, UPML slabs,
 *             ADE lists, excitation lists) in host memory.
 *   engine    Engine_CUDA: the Yee time stepping of Engine::IterateTS
 *             (FDTD/engine.cpp:255-274) with UPML, Lorentz/Drude ADE and
 *             excitation fused into the two half-step kernels, probes and the
 *             energy end criterion reduced on the device.
 *
 * Every function returns an int status: 0 = success, < 0 = error.  The text of
 * the last error of the calling thread is returned by fdtd_last_error().  No
 * function calls exit(); invalid input is reported, never trapped.
 *
 * Array layout used across the ABI ("reference form"): a field or coefficient
 * array of component n at node (x,y,z) lives at
 *     base[((n*Nx + x)*Ny + y)*Nz + z]          (z fastest, no padding)
 * which is the reference's FDTD_FLOAT**** [n][x][y][z] flattened.
 */
#ifndef WIPEMS_FDTD_H
#define WIPEMS_FDTD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ status */

#define FDTD_OK              0
#define FDTD_ERR_ARG        -1   /* invalid argument / size */
#define FDTD_ERR_CUDA       -2   /* CUDA runtime error */
#define FDTD_ERR_NOMEM      -3   /* host or device allocation failed */
#define FDTD_ERR_STATE      -4   /* call not valid in the object's state */
#define FDTD_ERR_UNSUPPORTED -5  /* feature not provided by this engine */
#define FDTD_ERR_TIMEOUT    -6   /* a bounded device wait gave up */
#define FDTD_ERR_NONFINITE  -7   /* energy reduction saw NaN/Inf */

/* Copies the calling thread's last error message (NUL terminated, truncated
 * to cap).  Returns the full message length. */
size_t fdtd_last_error(char* buf, size_t cap);

/* ------------------------------------------------------------------- scene */

typedef struct fdtd_scene_s* fdtd_scene_t;

/* Boundary condition codes, as openEMS::m_BC_type (openems.cpp:850-880). */
#define FDTD_BC_PEC 0
#define FDTD_BC_PMC 1
#define FDTD_BC_MUR 2   /* first-order Mur absorbing boundary */
#define FDTD_BC_PML 3

/* Mesh lines in drawing units (strictly increasing), unit = metres per
 * drawing unit (CSRectGrid::GetDeltaUnit, operator.cpp:806-812).
 * Replaces Operator::SetGeometryCSX + SetupCSXGrid (operator.cpp:821-836). */
int fdtd_scene_create(const double* lines_x, uint32_t nx,
                      const double* lines_y, uint32_t ny,
                      const double* lines_z, uint32_t nz,
                      double unit, fdtd_scene_t* out);
int fdtd_scene_destroy(fdtd_scene_t scene);

/* CSBackgroundMaterial (operator.cpp:825-830). */
int fdtd_scene_set_background(fdtd_scene_t s, double eps_r, double mue_r,
                              double kappa, double sigma);
/* bc[6] = xmin,xmax,ymin,ymax,zmin,zmax; pml_size[6] cells (PML_n), read
 * for PML faces only: every other face keeps openEMS's default size 8
 * (openems.cpp:101), which openEMS's UPML build still uses for the opposite
 * face's grading and the y/z slab ranges (operator_ext_upml.cpp:163,337).
 * pml_size may be null (every PML face 8 cells).
 * openEMS::SetupBoundaryConditions (openems.cpp:380-406). */
int fdtd_scene_set_boundary(fdtd_scene_t s, const int bc[6],
                            const uint32_t pml_size[6]);
/* Mur phase velocity per face (m/s; 0 = the speed of light in the
 * boundary material), <BoundaryCond MUR_PhaseVelocity[_xmin..]>
 * (openems.cpp:882-890). */
int fdtd_scene_set_mur_velocity(fdtd_scene_t s, const double v_phase[6]);
/* Gaussian pulse excitation signal, Excitation::SetupGaussianPulse
 * (excitation.cpp:55-62).  nr_ts = NumberOfTimesteps (signal length cap). */
int fdtd_scene_set_gauss_excite(fdtd_scene_t s, double f0, double fc,
                                uint32_t nr_ts);
/* Sinusoidal excitation of frequency f0, Excitation::SetupSinusoidal /
 * CalcSinusExcitation (excitation.cpp:65-71, 273-295): two periods of
 * sin(2 pi f0 t) (0 at t = 0), repeated with the period; the operator
 * shortens dT so that 1/f0 is a whole number of timesteps
 * (Operator::CalcECOperator, operator.cpp:1001-1007).  nr_ts > 0. */
int fdtd_scene_set_sinus_excite(fdtd_scene_t s, double f0, uint32_t nr_ts);
/* Dirac pulse (1 at timestep 1 only) and step (1 from timestep 0 on),
 * Excitation::SetupDiracPulse / SetupStepExcite and their Calc functions
 * (excitation.cpp:73-85, 179-218); both sample the probes every timestep
 * (Nyquist number 1).  f_max = <FDTD f_max>. */
int fdtd_scene_set_dirac_excite(fdtd_scene_t s, double f_max, uint32_t nr_ts);
int fdtd_scene_set_step_excite(fdtd_scene_t s, double f_max, uint32_t nr_ts);
/* Custom signal: `function` is an expression of the time t (seconds) with
 * the constants pi and e, Excitation::SetupCustomExcite /
 * CalcCustomExcitation (excitation.cpp:87-94, 233-271): nr_ts samples,
 * voltages at t = n dT and currents at t = (n + 1/2) dT, probes sampled at
 * the Nyquist number of f0.  Arithmetic (+ - * / % ^), parentheses and the
 * usual one- and two-argument functions are covered; comparisons, logical
 * operators and if() are refused. */
int fdtd_scene_set_custom_excite(fdtd_scene_t s, const char* function, double f0, double f_max,
                                 uint32_t nr_ts);
/* <FDTD OverSampling=...> (openems.cpp:830-832, default 4). */
int fdtd_scene_set_oversampling(fdtd_scene_t s, uint32_t oversampling);

/* Primitive boxes.  priority: the highest priority box containing a
 * coordinate wins (CSXCAD GetPropertyByCoordPriority); among equal
 * priorities the box added first wins.  Boxes contain their surface. */
int fdtd_scene_add_material(fdtd_scene_t s, int priority,
                            const double start[3], const double stop[3],
                            double eps_r, double kappa, double mue_r,
                            double sigma);
int fdtd_scene_add_metal(fdtd_scene_t s, int priority,
                         const double start[3], const double stop[3]);
/* Parallel R/C lumped element (Operator::Calc_LumpedElements,
 * operator.cpp:1535-1712).  R<0 or C<=0 mean "not given". */
int fdtd_scene_add_lumped(fdtd_scene_t s, int priority,
                          const double start[3], const double stop[3],
                          int direction, double R, double C, int caps);
/* Lumped RLC element (CSPropLumpedElement with an inductance or the series
 * type; Operator_Ext_LumpedRLC, operator_ext_lumpedRLC.cpp:112-486, and
 * Engine_Ext_LumpedRLC, engine_ext_lumpedRLC.cpp:83-145).  type:
 * FDTD_LE_PARALLEL (R || L || C; with L not given this is the element of
 * fdtd_scene_add_lumped), FDTD_LE_SERIES (R - L - C in series) or
 * FDTD_LE_INVALID (ignored, as the reference ignores it).  R, L, C < 0 mean
 * "not given".  The Gaussian's f0 + fc is the highest frequency used to
 * bound the edge's parasitic capacitance. */
#define FDTD_LE_INVALID (-1)
#define FDTD_LE_PARALLEL 0
#define FDTD_LE_SERIES 1
int fdtd_scene_add_lumped_rlc(fdtd_scene_t s, int priority,
                              const double start[3], const double stop[3],
                              int direction, int type, double R, double L,
                              double C, int caps);
/* Excitation box: exc_type 0 soft-E, 1 hard-E, 2 soft-H, 3 hard-H;
 * vec = weighted excitation per direction; delay in seconds
 * (operator_ext_excitation.cpp:134-220). */
int fdtd_scene_add_excitation(fdtd_scene_t s, int priority,
                              const double start[3], const double stop[3],
                              int exc_type, const double vec[3], double delay);
/* Drude / Lorentz material (CSPropLorentzMaterial): a material box with
 * eps_r/kappa/mue_r/sigma plus, per dispersion order o < order:
 * eps_plasma_f[o] (Hz), eps_relax_t[o] (s), eps_lor_pole_f[o] (Hz, 0 = Drude).
 * Read by Operator_Ext_LorentzMaterial::BuildExtension
 * (operator_ext_lorentzmaterial.cpp:117-438). */
int fdtd_scene_add_lorentz(fdtd_scene_t s, int priority,
                           const double start[3], const double stop[3],
                           double eps_r, double kappa, double mue_r,
                           double sigma, int order,
                           const double* eps_plasma_f,
                           const double* eps_relax_t,
                           const double* eps_lor_pole_f);
/* Drude / Lorentz material with both the electric and the magnetic
 * families of CSPropLorentzMaterial: per order o < order, eps_* act on the
 * E edges (from EC_C, the E-side ADE) and mue_plasma_f[o] (Hz),
 * mue_relax_t[o] (s), mue_lor_pole_f[o] (Hz, 0 = Drude) on the H edges
 * (from EC_L, the H-side ADE), operator_ext_lorentzmaterial.cpp:210-276.
 * Any of the six arrays may be NULL (all zeros: that family is off). */
int fdtd_scene_add_lorentz_material(fdtd_scene_t s, int priority,
                                    const double start[3], const double stop[3],
                                    double eps_r, double kappa, double mue_r,
                                    double sigma, int order,
                                    const double* eps_plasma_f,
                                    const double* eps_relax_t,
                                    const double* eps_lor_pole_f,
                                    const double* mue_plasma_f,
                                    const double* mue_relax_t,
                                    const double* mue_lor_pole_f);
/* Probe box: type 0 voltage (line integral, ProcessVoltage), type 1 current
 * (loop around a surface, ProcessCurrent); weight multiplies the integral;
 * norm_dir = normal direction of a current probe or -1.
 * openEMS::SetupProcessing (openems.cpp:480-560). */
int fdtd_scene_add_probe(fdtd_scene_t s, int type,
                         const double start[3], const double stop[3],
                         double weight, int norm_dir);

/* openEMS XML input (openEMS::ParseFDTDSetup, openems.cpp:756-936, and the
 * CSXCAD <ContinuousStructure> it embeds), the subset this engine covers:
 * <FDTD NumberOfTimesteps endCriteria OverSampling> with a Gaussian
 * <Excitation Type="0"> and <BoundaryCond> (PEC / PMC / MUR / PML_n or
 * codes, MUR_PhaseVelocity);
 * <RectilinearGrid DeltaUnit> with X/Y/ZLines; <BackgroundMaterial>; the
 * properties Material, Metal, LumpedElement (R, C, caps), Excitation,
 * ProbeBox (voltage / current / E / H field) and LorentzMaterial (order 1), each with
 * <Box Priority><P1/><P2/></Box> primitives.  Other content that changes
 * the simulation is refused with FDTD_ERR_UNSUPPORTED naming it; E / H
 * time-domain DumpBoxes are recorded (fdtd_scene_get_dump), other dumps and
 * mode-match probes are skipped (counted in `skipped`). */
typedef struct {
    uint32_t nr_ts;           /* NumberOfTimesteps */
    double   end_crit;        /* endCriteria (0 in the file -> 1e-6) */
    uint32_t oversampling;    /* OverSampling (0 = default) */
    int      excite_type;     /* <Excitation Type> */
    double   f0, fc;          /* Gaussian pulse */
    uint32_t num_properties, num_boxes, num_probes, skipped;
} fdtd_xml_info;

/* Time-domain field dumps the document asks for (<DumpBox DumpType="0|1"
 * DumpMode FileType SubSampling> with a Box; other dump types are skipped):
 * the box in drawing units, for the caller to snap and run with
 * fdtd_engine_dump_field at its interval. */
typedef struct {
    char     name[64];
    int      field;          /* FDTD_DUMP_E / FDTD_DUMP_H (DumpType 0 / 1) */
    int      interp;         /* DumpMode: FDTD_INTERP_NONE / NODE / CELL */
    int      file_type;      /* FileType: 0 VTK, 1 HDF5 */
    double   start[3], stop[3];
    uint32_t step[3];        /* SubSampling (1 = every line) */
} fdtd_scene_dump;
int fdtd_scene_num_dumps(fdtd_scene_t s, uint32_t* n);
int fdtd_scene_get_dump(fdtd_scene_t s, uint32_t k, fdtd_scene_dump* out);

int fdtd_scene_load_xml(const char* xml_text, fdtd_scene_t* out, fdtd_xml_info* info);
int fdtd_scene_load_xml_file(const char* path, fdtd_scene_t* out, fdtd_xml_info* info);

/* ---------------------------------------------------------------- operator */

typedef struct fdtd_operator_s* fdtd_operator_t;

/* Operator::CalcECOperator + extension builds (operator.cpp:973-1084) and
 * Excitation::buildExcitationSignal (openems.cpp:1124).  num_threads <= 0
 * picks the hardware concurrency (Operator_Multithread does the same). */
int fdtd_operator_build(fdtd_scene_t scene, int num_threads,
                        fdtd_operator_t* out);
int fdtd_operator_destroy(fdtd_operator_t op);

typedef struct {
    uint32_t num_lines[3];
    double   dT;                 /* Operator::GetTimestep */
    double   unit;               /* grid delta (m per drawing unit) */
    uint32_t nyquist;            /* Excitation::GetNyquistNum */
    uint32_t probe_interval;     /* max(1, Nyquist/OverSampling), openems.cpp:529 */
    uint32_t signal_length;      /* Excitation::GetLength */
    uint32_t max_excite_ts;      /* Excitation::GetMaxExcitationTimestep */
    uint32_t num_upml;           /* UPML slab extensions */
    uint32_t ade_order;          /* Lorentz/Drude dispersion order (0 = none) */
    uint32_t volt_exc_count;     /* Operator_Ext_Excitation::Volt_Count */
    uint32_t curr_exc_count;
    uint32_t num_probes;
    double   num_cells;          /* Operator::GetNumberCells (node count) */
} fdtd_operator_info;

int fdtd_operator_get_info(fdtd_operator_t op, fdtd_operator_info* info);

/* ---- reference-form operator description (what Engine_CUDA reads) ------ */

/* One Operator_Ext_UPML slab (operator_ext_upml.h:61-79): start/num_lines of
 * the slab in the full grid; the six coefficient arrays are
 * [3][nx][ny][nz] over the slab (z fastest). */
typedef struct {
    uint32_t start[3];
    uint32_t num_lines[3];
    const float* vv;   const float* vvfo; const float* vvfn;
    const float* ii;   const float* iifo; const float* iifn;
} fdtd_upml_desc;

/* One dispersion order of Operator_Ext_LorentzMaterial
 * (operator_ext_dispersive.h:47-53, operator_ext_lorentzmaterial.h): count
 * positions pos_x/y/z; coefficient arrays are [3][count] or NULL when the
 * corresponding *_on flag is 0. */
typedef struct {
    uint32_t count;
    const uint32_t* pos[3];
    int volt_on, curr_on, volt_lor_on, curr_lor_on;
    const float* v_int; const float* v_ext; const float* v_lor;
    const float* i_int; const float* i_ext; const float* i_lor;
} fdtd_ade_desc;

/* One Mur boundary face (Operator_Ext_Mur_ABC, operator_ext_mur_abc.cpp:
 * 88-205): the tangential voltages (components (ny+1)%3 and (ny+2)%3) on
 * line `line` of axis ny follow V = V'_shift - c V_line + c V_shift (old
 * values primed) from the neighbouring line `shift`, coefficients
 * c = (c0 dT - d) / (c0 dT + d) per (nP, nPP) position; active from
 * numTS >= start_ts. */
typedef struct {
    int      ny, top;
    uint32_t line, shift;
    uint32_t n_p, n_pp;        /* lines along (ny+1)%3 and (ny+2)%3 */
    const float* coef_p;       /* [n_p][n_pp] */
    const float* coef_pp;
    uint32_t start_ts;
} fdtd_mur_desc;

/* Lumped RLC edges (Operator_Ext_LumpedRLC, operator_ext_lumpedRLC.h:59-79):
 * per edge its node position and direction and the ADE coefficients.  Per
 * timestep, after the other post-update hooks:
 *   Il += i2v ilv Vd[n-1]                          (parallel inductor)
 *   Vd  = vvd (V - Il + vv2 Vd[n-2] + vj1 J[n-1] + vj2 J[n-2]);  V = Vd
 *   J   = ib0 (Vd - Vd[n-2]) - b1 ib0 J[n-1] - b2 ib0 J[n-2]      */
typedef struct {
    uint32_t count;
    const uint32_t* pos[3];
    const int* dir;
    const float* ilv; const float* i2v;
    const float* vv2; const float* vj1; const float* vj2; const float* vvd;
    const float* ib0; const float* b1; const float* b2;
} fdtd_rlc_desc;

/* Everything Engine_CUDA needs from an Operator after CalcECOperator. */
typedef struct {
    uint32_t num_lines[3];
    double   dT;
    const float* vv; const float* vi; const float* ii; const float* iv;
    uint32_t num_upml;
    const fdtd_upml_desc* upml;
    uint32_t num_ade_orders;
    const fdtd_ade_desc* ade;
    /* Operator_Ext_Excitation lists (operator_ext_excitation.h) */
    uint32_t volt_count;
    const uint32_t* volt_index[3];
    const uint16_t* volt_dir;
    const float*    volt_amp;
    const uint32_t* volt_delay;
    uint32_t curr_count;
    const uint32_t* curr_index[3];
    const uint16_t* curr_dir;
    const float*    curr_amp;
    const uint32_t* curr_delay;
    /* Excitation::GetVoltageSignal/GetCurrentSignal, GetLength */
    uint32_t signal_length;
    const float* signal_volt;
    const float* signal_curr;
    uint32_t signal_period_ts;   /* int(period/dT), 0 = not periodic */
    /* Mesh lines in drawing units and the grid delta (Operator::discLines,
     * GetGridDelta).  Optional (NULL / 0): needed only to compress graded
     * meshes with the factorized geometry. */
    const double* lines[3];
    double unit;
    /* Mur faces (Operator_Ext_Mur_ABC), in the order of the faces */
    uint32_t num_mur;
    const fdtd_mur_desc* mur;
    /* lumped RLC edges (NULL or count 0 = none) */
    const fdtd_rlc_desc* rlc;
} fdtd_op_desc;

/* Fills desc with pointers into op's host arrays (valid while op lives). */
int fdtd_operator_describe(fdtd_operator_t op, fdtd_op_desc* desc);

/* Snapped probe of the operator (ProcessIntegral after
 * DefineStartStopCoord).  type 0 voltage, 1 current, 2 E-field probe, 3
 * H-field probe (ProcessFieldProbe, Common/processfieldprobe.cpp:79-92: the
 * field at `start` -- main mesh for E, dual mesh and dual time for H --
 * without interpolation; three sample columns x, y, z in V/m or A/m). */
typedef struct {
    int      type;
    uint32_t start[3], stop[3];
    int      start_inside[3], stop_inside[3];
    int      norm_dir;
    double   weight;
    int      enabled;
} fdtd_probe_desc;

int fdtd_operator_get_probe(fdtd_operator_t op, uint32_t i,
                            fdtd_probe_desc* out);

typedef struct fdtd_engine_s* fdtd_engine_t;

/* -------------------------------------------------- compressed operator */

typedef struct fdtd_cop_s* fdtd_cop_t;

/* Host-side compression of a reference-form operator into per-node E and H
 * tuple indices (uint16 when the unique tuples of that half fit, else
 * uint32) plus coefficient tables holding vv/vi (ii/iv) and the fused UPML,
 * ADE and excitation terms -- the Operator_SSE_Compressed::CompressOperator
 * idea (operator_sse_compressed.cpp:120-176) applied per node and half-step.
 * Index arrays live in pinned host memory when a CUDA device is present.
 * Runs without a GPU.  fdtd_compress picks the mode automatically: exact on
 * uniform meshes (bit-identical coefficients), factorized geometry on graded
 * meshes when desc->lines is given (vi / iv rebuilt in-kernel as
 * VI * delta_n / A_n from per-axis arrays, within a few float ulps). */
int fdtd_compress(const fdtd_op_desc* desc, fdtd_cop_t* out);
/* mode: 0 = automatic, 1 = exact, 2 = factorized geometry */
int fdtd_compress_ex(const fdtd_op_desc* desc, int mode, fdtd_cop_t* out);
/* As fdtd_compress_ex, choosing the device axes: rotation r relabels the
 * grid cyclically so that device axis a is the operator's axis (a + r) % 3
 * (x -> y -> z -> x leaves the EC update and its FP32 operation order
 * unchanged, so the fields are bit-identical); -1 = automatic (the rotation
 * with the fewest padded nodes for 32-node z tiles, when it saves over 3 %).
 * fdtd_compress / fdtd_compress_ex choose automatically.  Everything the
 * engine takes or returns (probe boxes, field arrays, dump boxes, single
 * field values) stays in the operator's own axes. */
int fdtd_compress_rot(const fdtd_op_desc* desc, int mode, int rotation, fdtd_cop_t* out);
int fdtd_cop_destroy(fdtd_cop_t cop);

typedef struct {
    uint32_t num_lines[3];
    uint32_t num_tuples_e, num_tuples_h;
    uint32_t index_bytes_e, index_bytes_h;
    uint32_t padded_nz;
    uint32_t num_upml_nodes;
    uint32_t num_ade_nodes;
    int      geometry_factored;
    int      trim_e[3];       /* last line of the device axis is inert for E */
    uint64_t host_bytes;
    int      pinned;
    int      rotation;        /* device axis a = operator axis (a + rotation) % 3 */
    uint32_t device_lines[3]; /* the grid in device axes */
} fdtd_cop_info;

int fdtd_cop_get_info(fdtd_cop_t cop, fdtd_cop_info* info);
/* Expands the index + tables back to reference-form vv/vi/ii/iv -- the
 * coefficients the kernels apply, geometry factor included -- and the
 * per-node E/H flag words (any pointer may be NULL).  Test use. */
int fdtd_cop_expand(fdtd_cop_t cop, float* vv, float* vi, float* ii, float* iv,
                    uint32_t* flags_e, uint32_t* flags_h);
/* The extension coefficients of one half (0 = E, 1 = H) as the kernels apply
 * them, per node: ade = [9][Nx][Ny][Nz] (int[3], ext[3], lor[3] of the
 * Lorentz/Drude ADE: v_int / v_ext / v_lor or i_*), upml = [9][Nx][Ny][Nz]
 * (vvp|iip[3], vvfo|iifo[3], vvfn|iifn[3]); zero where a node has none.
 * Either pointer may be NULL.  With fdtd_cop_expand this rebuilds the whole
 * operator the engine steps on (test and inspection use). */
int fdtd_cop_expand_ext(fdtd_cop_t cop, int half, float* ade, float* upml);
/* The Lorentz/Drude ADE terms of one dispersion order (0..3) of one half as
 * the kernels apply them, ade = [9][Nx][Ny][Nz] as in fdtd_cop_expand_ext
 * (order 0 is the same array). */
int fdtd_cop_expand_ade(fdtd_cop_t cop, int half, int order, float* ade);

/* ------------------------------------------------------------------ engine */

typedef struct {
    int      device;          /* CUDA device ordinal */
    uint32_t max_timesteps;   /* sizes the probe/energy ring (0 = 100000) */
    uint32_t probe_interval;  /* samples at ts % interval == 0 (0 = off) */
    int      use_graphs;      /* capture chunks of interval steps */
    int      energy_on_probe; /* fuse the energy reduction into sample steps */
    int      tile_y;          /* kernel tile rows (0 = autotuned default) */
    int      x_chunk;         /* x planes per block (0 = chosen from the grid
                                 size by a wave model: 1, 2, 4, 8 or 16) */
    int      kernel;          /* 0 = default: the TMA-pipelined two-pass
                                     kernels (3),
                                 1 = direct-load kernels,
                                 2 = fused single-pass TMA kernel (E and H of
                                     a timestep in one x-march, double-
                                     buffered fields; not with Lorentz/Drude
                                     nodes or factorized geometry; fewer DRAM
                                     bytes but fewer resident blocks: measured
                                     slower than 3 on GB300 once the x-chunk
                                     is tuned),
                                 3 = TMA-pipelined two-pass kernels */
    int      stages;          /* TMA ring depth in x-planes, 3..8 (0 = 3) */
    double   end_crit;        /* > 0: the job stops on the device at the first
                                 sample whose energy is <= end_crit x the
                                 largest sampled energy, or at max_timesteps
                                 (openEMS::RunFDTD's end criterion,
                                 openems.cpp:1285-1314); needs probe_interval
                                 and energy_on_probe.  0 = off */
} fdtd_engine_opts;

/* Operator::CreateEngine for the CUDA engine: compresses the coefficient
 * arrays into a per-node uint16 (or uint32) index plus coefficient tables
 * (the Operator_SSE_Compressed idea, operator_sse_compressed.cpp:120-176,
 * extended by the UPML/ADE/excitation terms fused into the kernels) and
 * uploads everything to the device.  Field arrays start at zero
 * (Engine::Init, engine.cpp:49-57). */
int fdtd_engine_create(const fdtd_op_desc* desc, const fdtd_engine_opts* opts,
                       fdtd_engine_t* out);
/* The upload half of fdtd_engine_create: device arrays from an already
 * compressed operator (host -> device copies from pinned memory). */
int fdtd_engine_create_compressed(fdtd_cop_t cop, const fdtd_engine_opts* opts,
                                  fdtd_engine_t* out);
/* Engine::Reset + Engine::Init without reallocation: fields, UPML flux and
 * ADE states back to zero, numTS = 0, recorded samples dropped. */
int fdtd_engine_reset(fdtd_engine_t eng);
/* Engine::Reset (engine.cpp:98-106): frees device memory. */
int fdtd_engine_destroy(fdtd_engine_t eng);

/* Registers a probe (ProcessVoltage::CalcIntegral / ProcessCurrent::
 * CalcIntegral, processvoltage.cpp:43-47, processcurrent.cpp:93-168, or a
 * field probe) to be evaluated on the device at every sample step.  Must
 * precede the first iterate.  Returns the probe's first sample column in
 * *slot: one column per voltage / current probe, three per field probe
 * (field probes need the operator description's mesh lines). */
int fdtd_engine_add_probe(fdtd_engine_t eng, const fdtd_probe_desc* p,
                          uint32_t* slot);

/* Engine::IterateTS (engine.cpp:255-274). */
int fdtd_engine_iterate(fdtd_engine_t eng, uint32_t n_steps);
/* Engine::GetNumberOfTimesteps. */
/* fdtd_engine_iterate in two halves: _async queues the timesteps on the
 * engine's own stream and returns; _wait blocks until they are done and
 * reports their errors (numTS, done and samples are current after it).
 * Engines on different streams then run concurrently on the GPU; no other
 * call may touch the engine between the two. */
int fdtd_engine_iterate_async(fdtd_engine_t eng, uint32_t n_steps);
int fdtd_engine_wait(fdtd_engine_t eng);
/* *ready = 1 when no asynchronous iterate is outstanding or it has finished
 * on the device (fdtd_engine_wait then returns at once). */
int fdtd_engine_query(fdtd_engine_t eng, int* ready);
/* Frequency-domain probe accumulation on the device (ProcessIntegral::
 * Process, processintegral.cpp:154-168): on every timestep that is a
 * multiple of fd_interval (ts = 0 included), every probe's integral v
 * (weighted) is added as v * exp(-2 pi i f t) * 2 dT fd_interval for each
 * frequency f, t = numTS * dT (current probes: (numTS + 0.5) * dT).  The
 * reference's interval is Processing::AddFrequency's (processing.cpp:150-
 * 170): the operator's Nyquist number, lowered to CalcNyquistNum(f, dT) of
 * any higher frequency.  Set before the first iterate; not available in
 * batches.  read_fd returns [probe][frequency][re, im] and the number of
 * accumulated samples. */
int fdtd_engine_set_fd(fdtd_engine_t eng, const double* freqs, uint32_t nfreq,
                       uint32_t fd_interval);
int fdtd_engine_read_fd(fdtd_engine_t eng, double* re_im, uint32_t* samples);
/* Field dump from the device (ProcessFieldsTD / ProcessFields::CalcField,
 * Common/processfields_td.cpp:49-91, processfields.cpp:280-330, with the
 * interpolation of Engine_Interface_FDTD, engine_interface_fdtd.cpp:60-200):
 * E (V/m) or H (A/m) at the engine's current timestep on the mesh lines
 * start + i * step of a box (ProcessFields::CalcMeshPos with sub-sampling),
 * out[3][num0][num1][num2] as float.  out = NULL: only num[] is filled.
 * The file format (VTK / HDF5) is the caller's: wipems_gb300/dumps.py
 * writes legacy VTK rectilinear grids. */
#define FDTD_DUMP_E 0
#define FDTD_DUMP_H 1
#define FDTD_INTERP_NONE 0
#define FDTD_INTERP_NODE 1
#define FDTD_INTERP_CELL 2
typedef struct {
    int      field;               /* FDTD_DUMP_E or FDTD_DUMP_H */
    int      interp;              /* FDTD_INTERP_* */
    uint32_t start[3], stop[3];   /* mesh-line indices (either order) */
    uint32_t step[3];             /* sub-sampling per axis (0 = every line) */
} fdtd_dump_box;
int fdtd_engine_dump_field(fdtd_engine_t eng, const fdtd_dump_box* box,
                           float* out, uint64_t cap, uint32_t num[3]);

/* Checkpoint / resume (no counterpart in the reference, which has no
 * restart): every piece of the engine's device state -- fields, UPML flux,
 * Lorentz/Drude and Mur state, numTS, energy accumulators, the recorded
 * samples and frequency-domain sums -- as one host blob.  checkpoint with
 * buf = NULL only reports the size.  restore loads a blob into an engine
 * made from the same operator with the same options (before or after its
 * first iterate); stepping on from there gives the same results, bit for
 * bit, as stepping on from the checkpointed engine.  A server can use it to
 * take a job off the GPU and put it back later. */
int fdtd_engine_checkpoint(fdtd_engine_t eng, void* buf, uint64_t cap, uint64_t* size);
int fdtd_engine_restore(fdtd_engine_t eng, const void* buf, uint64_t size);
/* 1 once the engine's end criterion (opts.end_crit) stopped it, as of the
 * last iterate; numTS then stays at the stopping timestep. */
int fdtd_engine_done(fdtd_engine_t eng, int* done);
int fdtd_engine_num_timesteps(fdtd_engine_t eng, uint32_t* ts);

/* Number of recorded samples and the per-sample record layout:
 * ts[k], probe values [k][num_probes] (already multiplied by the weight),
 * energy[k] (eps0*sum V^2 + mu0*sum I^2, or -1 when not computed).
 * Reads all samples recorded so far (device -> host). */
int fdtd_engine_num_samples(fdtd_engine_t eng, uint32_t* n);
int fdtd_engine_read_samples(fdtd_engine_t eng, uint32_t first, uint32_t count,
                             uint32_t* ts, double* probe_values,
                             double* energy);

/* Engine_Interface_FDTD::CalcFastEnergy (engine_interface_fdtd.cpp:292-337)
 * computed now on the device. */
int fdtd_engine_energy(fdtd_engine_t eng, double* energy);

/* Copies all fields to host in reference form ([3][Nx][Ny][Nz]).  Either
 * pointer may be NULL.  Test / final-field use only. */
int fdtd_engine_get_fields(fdtd_engine_t eng, float* volt, float* curr);
/* Engine::GetVolt / GetCurr for one edge (device -> host read). */
int fdtd_engine_get_volt(fdtd_engine_t eng, uint32_t n, uint32_t x,
                         uint32_t y, uint32_t z, float* v);
int fdtd_engine_get_curr(fdtd_engine_t eng, uint32_t n, uint32_t x,
                         uint32_t y, uint32_t z, float* v);
/* Engine::SetVolt / SetCurr (engine.h:58-61): one field value. */
int fdtd_engine_set_volt(fdtd_engine_t eng, uint32_t n, uint32_t x,
                         uint32_t y, uint32_t z, float v);
int fdtd_engine_set_curr(fdtd_engine_t eng, uint32_t n, uint32_t x,
                         uint32_t y, uint32_t z, float v);
/* One probe integral of the current fields, unweighted, in the reference's
 * order and precision: a voltage line integral (type 0,
 * Engine_Interface_FDTD::CalcVoltageIntegral, engine_interface_fdtd.cpp:
 * 200-226) or a current loop (type 1, ProcessCurrent::CalcIntegral,
 * processcurrent.cpp:93-168).  For an openEMS processing that evaluates
 * integrals on its own schedule (Engine_Interface_CUDA). */
int fdtd_engine_probe_now(fdtd_engine_t eng, const fdtd_probe_desc* p,
                          double* value);

typedef struct {
    uint32_t num_tuples;      /* unique coefficient tuples after compression */
    uint32_t index_bytes;     /* 2 (uint16) or 4 (uint32) */
    uint32_t num_upml_nodes;  /* nodes inside UPML slabs */
    uint32_t num_ade_nodes;   /* nodes carrying ADE state */
    uint32_t padded_nz;       /* z row stride on the device */
    uint64_t device_bytes;    /* device memory held by the engine */
    uint32_t tile_y, x_chunk; /* kernel tiling in use */
    uint32_t kernel;          /* kernel family in use: 1, 2 or 3 as in
                                 fdtd_engine_opts.kernel */
} fdtd_engine_stats;

int fdtd_engine_get_stats(fdtd_engine_t eng, fdtd_engine_stats* st);

/* Runs n_steps timesteps launching each half-step kernel individually with
 * CUDA events around it on the engine stream; returns the mean duration of
 * one voltage-kernel and one current-kernel launch (ms).  The simulation
 * advances by n_steps exactly as fdtd_engine_iterate would. */
int fdtd_engine_profile_kernels(fdtd_engine_t eng, uint32_t n_steps,
                                double* ms_volt, double* ms_curr);

/* Device time of the last iterate call's kernels, measured with CUDA events
 * on the engine stream (ms) and the number of kernel launches it issued. */
int fdtd_engine_last_timing(fdtd_engine_t eng, double* ms, uint64_t* launches);

/* ----------------------------------------------------------------- batches */

/* Batched mode (no counterpart in the reference, which runs one simulation
 * per process): the jobs -- engines created as above, on one device, with
 * the TMA kernels -- advance together with one persistent kernel per
 * half-step and kernel variant over a flattened (job, tile) work list, each
 * job sampling its probes / energy at its own interval, the step sequence
 * replayed from a CUDA graph.  The engines stay owned by the caller and must
 * outlive the batch; per-job calls (read_samples, get_fields, reset) work
 * between batch iterations. */
typedef struct fdtd_batch_s* fdtd_batch_t;

typedef struct {
    int x_chunk;        /* x planes per work item (0 = chosen from the
                           batch's size by a wave model) */
    int stages;         /* TMA ring depth 3..8 (0 = 3) */
    int blocks_per_sm;  /* cap on resident blocks per SM (0 = occupancy);
                           -1 = no persistent blocks: one block per work
                           item, scheduled by the hardware */
    int graph_steps;    /* timesteps per captured graph (0 = 8, 1 = none) */
    int bin_mib;        /* L2 bins: jobs are packed into bins of at most this
                           many MiB of device state; each bin runs graph_steps
                           steps in a row so its data is re-read from L2
                           (0 = one bin with every job) */
    int chains;         /* each kernel-variant group is split into this many
                           job ranges (balanced by node count) that advance
                           as independent chains of kernels on their own
                           streams, so one chain's last wave overlaps the
                           others' work (0 = 1: one chain per group, the
                           groups in sequence) */
    int tile_y;         /* rows of the batched kernels' 32-lane tiles: 4 or 8
                           (0 = 8) */
} fdtd_batch_opts;

typedef struct {
    uint32_t num_jobs, num_groups, num_bins;
    uint64_t total_nodes;
    uint64_t work_items;
    uint32_t persistent_blocks;
    uint64_t device_bytes;
    double   last_ms;
    uint64_t last_launches;
    uint32_t x_chunk;   /* x planes per work item in use */
} fdtd_batch_stats;

int fdtd_batch_create(const fdtd_engine_t* engines, uint32_t n,
                      const fdtd_batch_opts* opts, fdtd_batch_t* out);
/* *ok = 1 when fdtd_batch_create would take the engine (two-pass TMA
 * kernels; no Mur face, lumped RLC edge or frequency-domain accumulation). */
int fdtd_batch_accepts(fdtd_engine_t eng, int* ok);
/* Advances every job by n_steps (each job's numTS moves by n_steps). */
int fdtd_batch_iterate(fdtd_batch_t batch, uint32_t n_steps);
int fdtd_batch_info(fdtd_batch_t batch, fdtd_batch_stats* stats);
int fdtd_batch_destroy(fdtd_batch_t batch);

/* ------------------------------------------------------------------ server */

/* Continuous-batching job server (no counterpart in the reference, which
 * runs one simulation per openEMS process).  Scenes are submitted at any
 * time; host worker threads build and compress their operators while the
 * GPU runs; one GPU thread retires jobs whose device end criterion fired,
 * admits built jobs while their device footprint fits the HBM budget, and
 * advances all resident jobs together in batched rounds (fdtd_batch_*).
 * A job stops at the same timestep, with the same samples and fields, as
 * it would alone.  All functions are thread-safe. */
typedef struct fdtd_server_s* fdtd_server_t;

enum {
    FDTD_JOB_QUEUED = 0,    /* waiting for a build worker */
    FDTD_JOB_BUILDING = 1,  /* operator build + compression on the host */
    FDTD_JOB_READY = 2,     /* built, waiting for device memory / a slot */
    FDTD_JOB_RUNNING = 3,   /* resident in HBM, advancing in the batch */
    FDTD_JOB_DONE = 4,      /* results on the host */
    FDTD_JOB_FAILED = 5
};

typedef struct {
    int      device;
    uint64_t hbm_budget;          /* bytes resident jobs may hold (0 = 90 % of free) */
    uint32_t max_active;          /* cap on resident jobs (0 = 256) */
    uint32_t round_steps;         /* timesteps per scheduling round (0 = 128) */
    int      build_workers;       /* concurrent operator builds (0 = auto) */
    int      build_threads_per_job; /* threads per operator build (0 = auto) */
    uint32_t batch_min_jobs;      /* with at least this many resident jobs,
                                     advance them as one persistent batch
                                     (fdtd_batch_*); otherwise (and with 0,
                                     the default) every job advances through
                                     its own engine, concurrently on its own
                                     stream */
    fdtd_batch_opts batch;        /* tiling of the batched kernels */
    uint32_t tile_share;          /* concurrent engines: each job's x-chunk is
                                     chosen as if it had 1/tile_share of the
                                     SMs (jobs overlap on their streams, so
                                     longer chunks with fewer halo planes
                                     pay); 0 = 4, 1 = the job alone */
} fdtd_server_opts;

typedef struct {
    double   end_crit;        /* energy decay stop, e.g. 1e-4 = -40 dB (0 = off:
                                 the job runs exactly max_timesteps; such jobs
                                 run as concurrent engines, not in batches) */
    uint32_t max_timesteps;   /* timestep cap (0 = the scene's NrTS) */
    uint32_t probe_interval;  /* 0 = the operator's Nyquist-derived interval */
    int      keep_fields;     /* copy the final fields to the host at retirement */
} fdtd_job_opts;

typedef struct {
    int      state;           /* FDTD_JOB_* */
    int      error;           /* status code of a failed job (message via fdtd_last_error) */
    uint32_t timesteps;       /* numTS at retirement */
    uint32_t num_samples, num_probes, probe_interval;  /* num_probes: sample columns */
    uint64_t nodes;           /* lines product */
    uint32_t num_lines[3];
    double   dT;              /* timestep (s) */
    uint64_t footprint;       /* device bytes reserved while resident */
    double   t_submit, t_built, t_admit, t_done;  /* s since fdtd_server_create */
} fdtd_job_status;

typedef struct {
    uint64_t jobs_submitted, jobs_admitted, jobs_done, jobs_failed;
    uint64_t rounds, rebuilds, kernel_launches;
    double   node_steps;      /* sum over finished jobs of nodes x timesteps */
    double   gpu_ms;          /* time with GPU work in flight: batch rounds by
                                 CUDA events, concurrent engines by the host
                                 clock while any has steps queued */
    uint64_t budget_bytes, used_bytes, peak_bytes;
    uint32_t active_jobs;
    int      last_error;
    double   elapsed_s;
} fdtd_server_stats;

int fdtd_server_create(const fdtd_server_opts* opts, fdtd_server_t* out);
/* Takes ownership of scene (do not destroy it afterwards). */
int fdtd_server_submit(fdtd_server_t srv, fdtd_scene_t scene, const fdtd_job_opts* opts,
                       uint64_t* job_id);
int fdtd_server_job_status(fdtd_server_t srv, uint64_t job_id, fdtd_job_status* st);
/* Blocks until the job (job_id = 0: every submitted job) is done or failed;
 * timeout_s <= 0 waits without limit. */
int fdtd_server_wait(fdtd_server_t srv, uint64_t job_id, double timeout_s);
/* Samples of a finished job: num_samples rows (see fdtd_job_status). */
int fdtd_server_read_samples(fdtd_server_t srv, uint64_t job_id, uint32_t* ts, double* vals,
                             double* energy);
int fdtd_server_get_fields(fdtd_server_t srv, uint64_t job_id, float* volt, float* curr);
/* The probe type (0..3) of each sample column of a built job (a field
 * probe fills three columns): types[num_probes] of fdtd_job_status. */
int fdtd_server_probe_types(fdtd_server_t srv, uint64_t job_id, int* types, uint32_t cap);
/* Drops a finished job's host results. */
int fdtd_server_release(fdtd_server_t srv, uint64_t job_id);
int fdtd_server_get_stats(fdtd_server_t srv, fdtd_server_stats* st);
/* Stops the threads; queued and running jobs are abandoned. */
int fdtd_server_destroy(fdtd_server_t srv);

/* ---------------------------------------------------- allocation-free path */

/* Energy eps0*sum(V^2) + mu0*sum(I^2) over x < Nx-1, y < Ny-1, z < Nz-1 of
 * caller-owned device fields -- the quantity fdtd_engine_energy returns --
 * for callers that must not allocate device memory (a fixed memory budget,
 * a real-time loop that may not touch the allocator, an embedding
 * application whose allocator is off limits).  No counterpart in the
 * reference: it has no device code.
 *   volt, curr   device arrays [3][Nx][Ny][z_pitch] (z fastest)
 *   num_lines    {Nx, Ny, Nz};  z_pitch >= Nz
 *   stream       cudaStream_t to launch on (NULL = default stream)
 *   energy       device pointer receiving one double
 * The per-plane partial sums live in a static device array of 4096 planes
 * (64 KB, held by every GPU that loads the library until exit); Nx-1 above
 * 4096 is rejected with FDTD_ERR_ARG.  Calls no cudaMalloc / cudaFree.  The
 * first call on a device looks the array up with cudaGetSymbolAddress, so
 * make that first call before any stream capture.  All calls share the
 * array: calls that overlap on the GPU race. */
int fdtd_field_energy_static(const float* volt, const float* curr,
                             const uint32_t num_lines[3], uint32_t z_pitch,
                             void* stream, double* energy);

#ifdef __cplusplus
}
#endif

#endif /* WIPEMS_FDTD_H */
