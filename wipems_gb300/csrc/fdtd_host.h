// Host-side data structures of the FDTD operator (setup-time C++).
//
// The scene is the stand-in for the CSXCAD geometry database: rectilinear
// mesh lines plus priority-ordered boxes.  The operator holds the
// reference-form coefficient arrays that openEMS's Operator and its
// extensions hold after CalcECOperator (FDTD/operator.h:285-288,
// extensions/operator_ext_upml.h:61-79, operator_ext_lorentzmaterial.h,
// operator_ext_excitation.h).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/wipems_fdtd.h"

namespace wipems {

// tools/constants.h:21-27
constexpr double kEps0 = 8.85418781762e-12;
constexpr double kMue0 = 1.256637062e-6;
constexpr double kC0 = 299792458;
constexpr double kZ0 = 376.730313461;
constexpr double kPi = 3.141592653589793238462643383279;

enum PrimKind { PK_MATERIAL = 1, PK_METAL = 2, PK_LUMPED = 3, PK_EXCITATION = 4, PK_PROBE = 5 };

constexpr int kMaxDispOrder = 4;

struct Prim {
    int kind = 0;
    int priority = 0;
    double start[3] = {0, 0, 0}, stop[3] = {0, 0, 0};
    double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};  // ordered bounds
    // material / lorentz
    double eps = 1, kappa = 0, mue = 1, sigma = 0;
    bool lorentz = false;
    int disp_order = 0;
    double eps_plasma_f[kMaxDispOrder] = {0, 0, 0, 0};
    double eps_relax_t[kMaxDispOrder] = {0, 0, 0, 0};
    double eps_lor_pole_f[kMaxDispOrder] = {0, 0, 0, 0};
    double mue_plasma_f[kMaxDispOrder] = {0, 0, 0, 0};
    double mue_relax_t[kMaxDispOrder] = {0, 0, 0, 0};
    double mue_lor_pole_f[kMaxDispOrder] = {0, 0, 0, 0};
    // lumped element
    int ny = 2;
    double R = -1, C = -1, L = -1;
    int le_type = 0;  // FDTD_LE_PARALLEL / SERIES / INVALID
    bool caps = false;
    // excitation
    int exc_type = 0;
    double exc_vec[3] = {0, 0, 0};
    double delay = 0;
    // probe
    int probe_type = 0;
    double weight = 1;
    int norm_dir = -1;
};

}  // namespace wipems

namespace wipems {
// a time-domain field dump of the scene (<DumpBox>), applied by the caller
struct DumpSpec {
    std::string name;
    int field = 0;   // 0 = E, 1 = H (DumpType 0 / 1)
    int interp = 0;  // DumpMode: 0 none, 1 node, 2 cell
    int file_type = 0;
    double start[3] = {0, 0, 0}, stop[3] = {0, 0, 0};
    uint32_t step[3] = {1, 1, 1};
};
}  // namespace wipems

struct fdtd_scene_s {
    std::vector<double> lines[3];
    double unit = 1;
    double bg_eps = 1, bg_mue = 1, bg_kappa = 0, bg_sigma = 0;
    int bc[6] = {0, 0, 0, 0, 0, 0};
    uint32_t pml_size[6] = {8, 8, 8, 8, 8, 8};  // openEMS default (openems.cpp:101)
    double mur_vph[6] = {0, 0, 0, 0, 0, 0};
    double f0 = 0, fc = 0;
    // Excitation::ExciteTypes (excitation.h:28): 0 Gaussian pulse,
    // 1 sinusoid, 2 Dirac pulse, 3 step, 10 custom function of t; f_max is
    // the Dirac / step / custom <FDTD f_max> (recorded, it changes nothing on
    // this path)
    int excite_type = 0;
    double f_max = 0;
    std::string exc_function;  // the custom signal's expression
    bool have_excite = false;
    uint32_t nr_ts = 0;
    uint32_t oversampling = 4;
    std::vector<wipems::Prim> prims;
    std::vector<wipems::DumpSpec> dumps;
};

namespace wipems {

struct UpmlSlab {
    uint32_t start[3];
    uint32_t num_lines[3];
    // [3][nx][ny][nz]
    std::vector<float> vv, vvfo, vvfn, ii, iifo, iifn;
};

struct AdeOrder {
    uint32_t count = 0;
    std::vector<uint32_t> pos[3];
    bool volt_on = false, curr_on = false, volt_lor_on = false, curr_lor_on = false;
    std::vector<float> v_int, v_ext, v_lor, i_int, i_ext, i_lor;  // [3][count]
};

struct MurFace {
    int ny = 0, top = 0;
    uint32_t line = 0, shift = 0;
    uint32_t n[2] = {0, 0};
    std::vector<float> cp, cpp;  // [n[0]][n[1]]
    uint32_t start_ts = 0;
};

// Operator_Ext_LumpedRLC's arrays (operator_ext_lumpedRLC.h:59-79)
struct RlcList {
    std::vector<uint32_t> pos[3];
    std::vector<int> dir;
    std::vector<float> ilv, i2v, vv2, vj1, vj2, vvd, ib0, b1, b2;
    size_t size() const { return dir.size(); }
};

struct ExcList {
    std::vector<uint32_t> index[3];
    std::vector<uint16_t> dir;
    std::vector<float> amp;
    std::vector<uint32_t> delay;
};

}  // namespace wipems

struct fdtd_operator_s {
    uint32_t N[3] = {0, 0, 0};
    double unit = 1;
    std::vector<double> lines[3];
    double dT = 0;
    // reference-form coefficient arrays [3][Nx][Ny][Nz]
    std::vector<float> vv, vi, ii, iv;
    std::vector<wipems::UpmlSlab> upml;
    std::vector<wipems::AdeOrder> ade;
    wipems::ExcList volt_exc, curr_exc;
    std::vector<float> sig_volt, sig_curr;
    uint32_t signal_length = 0;
    uint32_t signal_period_ts = 0;  // 0: not periodic
    uint32_t nyquist = 0;
    uint32_t probe_interval = 1;
    uint32_t max_excite_ts = 0;
    std::vector<fdtd_probe_desc> probes;
    // descriptor scratch kept alive for fdtd_operator_describe
    std::vector<fdtd_upml_desc> upml_desc;
    std::vector<fdtd_ade_desc> ade_desc;
    std::vector<wipems::MurFace> mur;
    std::vector<fdtd_mur_desc> mur_desc;
    wipems::RlcList rlc;
    fdtd_rlc_desc rlc_desc{};
};

namespace wipems {
void set_error(const std::string& msg);
const std::string& last_error();  // this thread's last error message
// x planes per block for a grid of N[3] lines that gets about 1/share of the
// SMs of `device` (the wave model of the engine's automatic choice); 0 when
// the device cannot be queried
int engine_auto_x_chunk(const uint32_t N[3], int device, unsigned share);
}
