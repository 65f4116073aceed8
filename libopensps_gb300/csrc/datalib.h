// Data libraries in OpenSPS's standard format (version 1): a data root with `opensps-data.json`, each library a
// `libraries/<kind>/<name>/manifest.json` plus one raw little-endian array per file (doc/DATA_FORMAT.md section 2;
// the reader src/io/opensps_datalib.f90, the JSON parser src/io/opensps_json.f90). Host code only.
#pragma once
#include <string>
#include <utility>
#include <vector>

namespace sps {

// A JSON value (the six kinds of the grammar; objects keep their keys in order).
struct JVal {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    double num = 0.0;
    bool b = false;
    std::string str;
    std::vector<JVal> items;          // array items, object values
    std::vector<std::string> keys;    // object keys
    const JVal *get(const std::string &k) const;
};
bool json_parse(const std::string &text, JVal &out, std::string &err);

// OPENSPS_DATA_FORMAT (or FSPS_DATA_FORMAT): "auto" (default: a library is read from the standard layout when its
// manifest exists), "standard" (always; a missing manifest is an error), "legacy" (never: this package's own layout).
enum DataFormat { DF_AUTO = 0, DF_LEGACY = 1, DF_STANDARD = 2, DF_BAD = -1 };
DataFormat data_format_from_env();
bool datalib_root_is_standard(const std::string &root);
// whether kind/name (name may carry ":axis=value" selections) is read from the standard layout
bool datalib_available(const std::string &root, const std::string &kind, const std::string &name);

// One opened library (datalib_open, opensps_datalib.f90:145-220). Every call returns 0 or a status with `err` set.
struct DataLib {
    std::string dir, kind, name;
    JVal doc;
    std::vector<std::pair<std::string, std::string>> sel;   // axis selections of "name:axis=value,..."
    int open(const std::string &root, const std::string &kind, const std::string &spec, std::string &err);
    const JVal *meta(const std::string &key) const;
    bool has_axis(const std::string &axis) const;
    bool has_array(const std::string &name) const;
    int axis_len(const std::string &axis, long long &n, std::string &err) const;
    int axis_values(const std::string &axis, std::vector<double> &v, std::string &err) const;
    int array_len(const std::string &name, long long &n, std::string &err) const;
    // array `name` ends with `axes` of lengths `dims` (any extra leading axes resolved by the selections or the
    // axis's "default"); the element offset of the selected block (datalib_check_array :346-397)
    int check_array(const std::string &name, const std::vector<std::string> &axes, const std::vector<long long> &dims,
                    long long &offset, std::string &err) const;
    int read_real(const std::string &name, long long n, long long offset, std::vector<double> &out, std::string &err) const;
    int read_int(const std::string &name, long long n, long long offset, std::vector<long long> &out, std::string &err) const;

  private:
    int fail(std::string &err, const std::string &msg) const;
    int select_index(const std::string &axis, const std::string &value, int &idx, std::string &err) const;
    int read_desc(const JVal &d, const std::string &what, long long n, long long offset, bool integer,
                  std::vector<double> *outf, std::vector<long long> *outi, std::string &err) const;
};

// ---- the library kinds this path reads, on the model's wavelength grid (increasing, Angstrom)

// ssp/<name> (read_bpass_standard, src/io/opensps_io.f90:3131-3155): wavelength, log_age, Z (or [Fe/H]) axes,
// metadata solar_metallicity, spectra [Z, log_age, wavelength], stellar_mass [Z, log_age]; log L_bol per grid point
// is the trapezoid integral of the spectrum over frequency (ssp_gen's BPASS branch, opensps_ssp.f90:203-218).
// Nebular lines, when the library carries them: `line_luminosity` [Z, log_age, line_wavelength].
struct SspLibrary {
    std::vector<double> lam, log_age, zlegend, spec, mass, lbol, line_lambda, line_lum;
    double zsol = 0.0;
    int nspec = 0, nt = 0, nz = 0, nline = 0;
};
int std_load_ssp(const std::string &root, const std::string &spec, SspLibrary &out, std::string &err);

// dust_emission/<DL07|THEMIS> (read_dust_emission, opensps_io.f90:991-1060): per q_PAH and U_min component the
// template interpolated linearly (extrapolated beyond the table) at the grid's pixels from the one holding 1 um up,
// zero below. tab is float, (2 numin x nqpah) columns of nspec pixels, column (2 u + c) nqpah + q.
int std_load_dust_emission(const std::string &root, const std::string &spec, const std::vector<double> &lam,
                           std::vector<double> &qpah, std::vector<double> &umin, std::vector<double> &tab,
                           std::string &err);

// agn_torus/clumpy (load_agn_dust_models, opensps_io.f90:1099-1157): 9 optical depths; each template interpolated
// in log10(f + SAFE_FLOOR) against log10 lambda over the grid pixels within the table's range. tab: ntau x nspec.
int std_load_agn(const std::string &root, const std::vector<double> &lam, std::vector<double> &tau,
                 std::vector<double> &tab, std::string &err);

// nebular/<isoc>_<nodust|dust> (load_nebular_grid / read_nebular_standard, opensps_io.f90:749-827,910-933): the
// continuum [logZ (11), age (10), logU (7), wavelength] as log10(f + 1e-95) interpolated linearly (extrapolated beyond
// the table) at the grid's pixels; tab is nspec x 11 x 10 x 7, pixel fastest, then logZ, age, logU (nebem_cont(j, z,
// a, u)); lage = log10 of the ages. The lines array is not read (this path's lines are the SSP library's).
constexpr int NEB_NZ = 11, NEB_NAGE = 10, NEB_NU = 7;
int std_load_nebular(const std::string &root, const std::string &spec, const std::vector<double> &lam,
                     std::vector<double> &logz, std::vector<double> &lage, std::vector<double> &logu,
                     std::vector<double> &tab, std::string &err);

// attenuation/smc_bar and attenuation/dirty (load_attenuation_curves, src/io/opensps_io.f90:2079-2234): the SMC bar's
// A(lambda) / A(V) over its wavelength axis, or the dusty environments' optical depths [structure (2), tau_v (18),
// model (6), wavelength (25)]; each curve interpolated linearly at the grid's pixels inside the table's range, its
// first value below it and zero above. tab: the smc_bar curve (nspec), or the dirty curves (2 x 18 x 6 curves of
// nspec pixels, in the array's order: structure, then tau_v, then model).
constexpr int WG_NSTRUCT = 2, WG_NTAU = 18, WG_NMODEL = 6, WG_NLAM = 25;
int std_load_attenuation(const std::string &root, const std::string &name, const std::vector<double> &lam,
                         std::vector<double> &tab, std::string &err);

// filters/<name> (read_filter_library, opensps_io.f90:1247-1318, then filters_build with point resampling,
// src/spectra/opensps_filters.f90:395-500): bands nb x nspec normalised to int T / lambda = 1 on the grid, their
// pivot wavelengths and names; a filter with a calibration {lambda_ref, exponent} is then divided by
// int (lambda / lambda_ref)^exponent T / lambda (apply_standard_filter_calibration, opensps_io.f90:1465-1500).
int std_load_filters(const std::string &root, const std::string &spec, const std::vector<double> &lam,
                     std::vector<double> &bands, std::vector<double> &pivot, std::vector<std::string> &names,
                     std::string &err);

}  // namespace sps
