// config.cpp — reads a reference parameter file into wave_config.
//
// Same file rules as Configuration::readFromFile (Configuration/Configuration.cpp:45-100):
// one KEY=VALUE per line, keys case-insensitive, a line starting with '#' is
// skipped and a later '#' ends the value; a repeated key overwrites the
// earlier one. Values are read like Configuration::get<T> (Configuration.hpp:95-108):
// stream extraction of the leading token ("0;" reads as 0).
#include <algorithm>
#include <cctype>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "wave_internal.h"

namespace wave {

namespace {

std::string lower(std::string s)
{
    std::transform(s.begin(), s.end(), s.begin(), [](unsigned char c) { return static_cast<char>(std::tolower(c)); });
    return s;
}

template <class T>
bool get(const std::map<std::string, std::string>& m, const char* key, T& out)
{
    auto it = m.find(lower(key));
    if (it == m.end()) return false;
    std::istringstream in(it->second);
    T v{};
    in >> v;
    if (in.fail()) return false;
    out = v;
    return true;
}

// gridConfigurationFilename: rows "interface dhFactor FDorder", '#' lines and
// blank lines skipped (Common::readColumnFromFile, Common/Common.hpp:27-60).
// The name is taken as given (relative to the working directory, as the
// reference does), else relative to the parameter file's folder or its parent.
int read_grid_config(const std::string& name, const char* paramPath, wave_config& c, std::string& err)
{
    std::string dir(paramPath);
    size_t sl = dir.find_last_of('/');
    dir = sl == std::string::npos ? std::string(".") : dir.substr(0, sl);
    const std::string tries[3] = {name, dir + "/" + name, dir + "/../" + name};
    std::ifstream f;
    for (const std::string& t : tries) {
        f.open(t);
        if (f.is_open()) break;
        f.clear();
    }
    if (!f.is_open()) {
        err = "Could not open grid configuration " + name;
        return WAVE_ERR_IO;
    }
    std::string line;
    int rows = 0, lineNo = 0;
    while (std::getline(f, line)) {
        ++lineNo;
        if (line.empty() || line[0] == '#' || std::all_of(line.begin(), line.end(), [](unsigned char ch) { return std::isspace(ch); }))
            continue;
        std::istringstream in(line);
        std::vector<int> v;
        int x;
        while (in >> x) v.push_back(x);
        if (v.size() < 2 || (c.useVariableFDoperators && v.size() < 3)) {
            err = "line " + std::to_string(lineNo) + " in file " + name + " has too few columns";
            return WAVE_ERR_ARG;
        }
        if (rows == WAVE_MAX_GRID_LAYERS) {
            err = "more than " + std::to_string(WAVE_MAX_GRID_LAYERS) + " layers in " + name;
            return WAVE_ERR_ARG;
        }
        c.gridInterface[rows] = v[0];
        c.gridDHFactor[rows] = v[1];
        c.gridFDOrder[rows] = v.size() > 2 ? v[2] : c.spatialFDorder;
        ++rows;
    }
    c.gridLayers = rows;
    return WAVE_OK;
}

} // namespace

int parse_config_file(const char* path, wave_config* cfg, std::string& err)
{
    std::ifstream f(path);
    if (!f.good()) {
        err = std::string("Configuration file ") + path + " was not found";
        return WAVE_ERR_IO;
    }
    std::map<std::string, std::string> m;
    std::string line;
    while (std::getline(f, line)) {
        size_t end = line.size();
        size_t c = line.find('#');
        if (c != std::string::npos) {
            if (c == 0) continue;
            end = c;
        }
        size_t e = line.find('=');
        if (e == std::string::npos) continue;
        m[lower(line.substr(0, e))] = line.substr(e + 1, end > e ? end - e - 1 : 0);
    }
    wave_config c{};
    std::string dim, eq;
    if (!get(m, "dimension", dim) || !get(m, "equationType", eq)) {
        err = "Parameter dimension / equationType: Not found in Configuration file!";
        return WAVE_ERR_ARG;
    }
    dim = lower(dim);
    eq = lower(eq);
    if (dim == "2d") c.dimension = 2;
    else if (dim == "3d") c.dimension = 3;
    else { err = "Unkown dimension"; return WAVE_ERR_ARG; }
    static const std::map<std::string, int> eqs = {
        {"acoustic", WAVE_EQ_ACOUSTIC}, {"elastic", WAVE_EQ_ELASTIC}, {"viscoelastic", WAVE_EQ_VISCOELASTIC},
        {"sh", WAVE_EQ_SH}, {"viscosh", WAVE_EQ_VISCOSH}, {"tmem", WAVE_EQ_TMEM}, {"emem", WAVE_EQ_EMEM},
        {"viscotmem", WAVE_EQ_VISCOTMEM}, {"viscoemem", WAVE_EQ_VISCOEMEM}};
    auto it = eqs.find(eq);
    if (it == eqs.end()) { err = "Unkown type"; return WAVE_ERR_ARG; }
    c.equation = it->second;
    long long nx = 0, ny = 0, nz = 1;
    bool ok = get(m, "NX", nx) && get(m, "NY", ny) && get(m, "NZ", nz) && get(m, "DH", c.DH) &&
              get(m, "DT", c.DT) && get(m, "T", c.T) && get(m, "spatialFDorder", c.spatialFDorder);
    if (!ok) { err = "a mandatory key (NX, NY, NZ, DH, DT, T, spatialFDorder) is missing"; return WAVE_ERR_ARG; }
    c.NX = nx; c.NY = ny; c.NZ = c.dimension == 2 ? 1 : nz;
    c.FreeSurface = 0; get(m, "FreeSurface", c.FreeSurface);
    c.DampingBoundary = 0; get(m, "DampingBoundary", c.DampingBoundary);
    c.BoundaryWidth = 0; get(m, "BoundaryWidth", c.BoundaryWidth);
    c.DampingCoeff = 8.0; get(m, "DampingCoeff", c.DampingCoeff);
    c.NPower = 4.0; get(m, "NPower", c.NPower);
    c.CenterFrequencyCPML = 5.0; get(m, "CenterFrequencyCPML", c.CenterFrequencyCPML);
    c.VMaxCPML = 3500.0; get(m, "VMaxCPML", c.VMaxCPML);
    c.numRelaxationMechanisms = 0; get(m, "numRelaxationMechanisms", c.numRelaxationMechanisms);
    if (c.numRelaxationMechanisms < 0) c.numRelaxationMechanisms = 0;
    const char* rk[4] = {"relaxationFrequency", "relaxationFrequency2", "relaxationFrequency3", "relaxationFrequency4"};
    for (int l = 0; l < 4; ++l) { c.relaxationFrequency[l] = 0.0; get(m, rk[l], c.relaxationFrequency[l]); }
    c.useStencilMatrix = 0; get(m, "useStencilMatrix", c.useStencilMatrix);
    c.edgeOrderReduction = 1; get(m, "edgeOrderReduction", c.edgeOrderReduction);
    c.useVariableGrid = 0; get(m, "useVariableGrid", c.useVariableGrid);
    c.useVariableFDoperators = 0; get(m, "useVariableFDoperators", c.useVariableFDoperators);
    if (c.useVariableGrid || c.useVariableFDoperators) {
        std::string grid;
        if (!get(m, "gridConfigurationFilename", grid)) {
            err = "Parameter gridConfigurationFilename: Not found in Configuration file!";
            return WAVE_ERR_ARG;
        }
        int rc = read_grid_config(grid, path, c, err);
        if (rc != WAVE_OK) return rc;
    }
    *cfg = c;
    return WAVE_OK;
}

} // namespace wave
