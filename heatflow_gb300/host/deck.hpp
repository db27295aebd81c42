// Input decks and output formats of HeatFlow, host side in C++: param.in / mat.in / system.in
// readers (src/heatflow/mod_inputs.f90 read_param :204-360, check_param :366-596, read_system
// :602-649, read_mat :654-721, val :819-826), the material table (src/heatflow/mod_material.f90
// :54-267), the restart/result file format (mod_output.f90 final_print :207-238,
// mod_init_evolve.f90 read_temp_file :66-140) and the sub-box log record (mod_output.f90 :57-113).
// The result is an hf_problem for the C ABI of libheatflow_gb300.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "heatflow_gb300.h"

namespace hfhost {

// The reference prints a message and executes `stop` for these inputs.
struct InputError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct Param {
  int64_t iverb = 1, ntime = 10, heattime = 0, write_every = 1, iboundary = 1, icattaneo = 1,
          isteady = 0, temp_dep_prop = 0;
  int64_t start_ix = 1, end_ix = 0, start_iy = 1, end_iy = 0, start_iz = 1, end_iz = 0;
  double time_step = 1.0, freq = 1.0, power_in = 0.0, t_system = 300.0, t_bath = 0.0,
         t_bath_cg = 0.0, br = 1.0;
  double kappa_bound = 0.0, kb[6] = {0, 0, 0, 0, 0, 0};      // x1, Nx, y1, Ny, z1, Nz
  double t_bath_face[6] = {0, 0, 0, 0, 0, 0};                // x1, x2, y1, y2, z1, z2
  bool check_sparse_full = false, check_stability = false, write_to_txt = false,
       percentage_completion = false, test_run = false, input_temp_dis = false,
       full_restart = false, t_bath_cc = false;
  std::string run_name = "default", periodic_text, cg_dir;
  bool periodic[3] = {false, false, false};
  bool cg[6] = {false, false, false, false, false, false};   // -x, +x, -y, +y, -z, +z
};

struct Material {
  int64_t index = 0;
  double heat_capacity = 0, h_conv = 0, kappa = 0, kappa3D = 0, rho = 0, sound_speed = 0, tau = 0,
         em = 0;
};

struct System {
  int64_t nx = 0, ny = 0, nz = 0;
  double lx = 0, ly = 0, lz = 0;
  std::vector<int64_t> imaterial, iheater;   // x fastest
};

Param read_param(const std::string& text);
std::vector<Material> read_mat(const std::string& text);
System read_system(const std::string& text);
Material material(int64_t imaterial, const std::vector<Material>& mats);

// Temperature tables of the materials (TempDepProp = 1): the per-material file
// ./inputs/MatTable<imaterial> that ChangeProp looks for (mod_tempdep.f90:44-55), in the format of
// the reference's test/data/tempdep.in -- one row per line, four numbers: T (ascending), kappa,
// rho, heat capacity.  Laid out for hf_set_property_tables: table k is rows[4*offsets[k] ..
// 4*offsets[k+1]), materials[k] its material index, cell_table the table of each cell or -1.
struct PropertyTables {
  std::vector<int64_t> materials;
  std::vector<int32_t> offsets;
  std::vector<double> rows;
  std::vector<int32_t> cell_table;
  int32_t ntables() const { return offsets.empty() ? 0 : (int32_t)offsets.size() - 1; }
};
// One table's rows (4 values each); InputError on a ragged row, fewer than two rows, or
// temperatures that do not ascend.
std::vector<double> parse_property_table(const std::string& text, const std::string& name);
// Tables of every material of the grid that has a MatTable<imaterial> file in inputs_dir
// (materials in ascending index order); materials without a file keep fixed properties.
PropertyTables load_material_tables(const std::string& inputs_dir, const System& sys);

// A deck's problem: per-cell arrays owned here, `prob` points into them.
struct Deck {
  Param param;
  std::vector<Material> mats;
  System sys;
  std::vector<double> kappa, rho, heat_capacity, tau, em;
  hf_problem prob{};
  PropertyTables tables;   // loaded when TempDepProp = 1
  int64_t ncells() const { return sys.nx * sys.ny * sys.nz; }
};
// read_all_files on in-memory decks (mod_inputs.f90:116-196) + set_global_variables' per-cell part
// (mod_setup.f90:53-68).
void build_deck(Deck& deck, const std::string& param_text, const std::string& mat_text,
                const std::string& system_text);
std::string read_text_file(const std::string& path, const std::string& missing_message);

// final_print's layout: 6 values per line, ES16.8 each followed by one blank, two empty lines.
std::string format_temp_file(const double* v, int64_t n);
// read_temp_file: exactly `na` values (errors as the reference's).
std::vector<double> parse_temp_file(const std::string& text, int64_t na);
// One sub-box log record: the time in single precision, then the box values x fastest.
std::string format_record(double time, const double* v, int64_t n);
// First ./outputs/output_<RunName>_NN (NN from 00) that does not exist (last_log, :187-201).
std::string next_log_name(const std::string& outdir, const std::string& run_name);

// Records data_write appends to the sub-box log after step `itime` (mod_output.f90:79-113): one
// when the log is opened at itime = 1, and one more whenever _WriteToTxt is set and
// mod(itime, write_every) = 0 -- so with write_every = 1, step 1 is logged twice.  Test runs log
// nothing.
int records_after(const Param& p, int64_t itime);

// The deck's problem as JSON (parsed values; the per-cell arrays as lists), for comparisons.
std::string problem_json(const Deck& deck);

}  // namespace hfhost
