// lbm_gb300 -- the reference's io layer (namespace lbm::io) for the drop-in C++ API:
//
//   Config                 io/configuration.h:15-145   config file + command line
//   parse_scenario_file    io/scenario.h:131-188       XML scenario -> Domain
//   read_vtk_point_file    io/vtk.hpp:93-157           legacy-VTK fluid mask -> Domain
//   write_vtk_file         io/vtk.hpp:42-89            <dir>/<name>.<t>.vts from device moments
//   VtkWriter              (extension)                 the same files, written on a background
//                                                      thread while the time loop runs on
//
// No boost, pugixml or VTK: the config file, the XML subset the scenarios use (prolog, comments,
// elements, quoted attributes) and the legacy STRUCTURED_POINTS format are parsed here, and the
// VTS StructuredGrid is written here (binary DataArrays, base64 with a UInt32 byte count). Node
// and attribute names, face names, defaults and error messages follow the reference; errors are
// std::logic_error, as there.
#pragma once

#include <cctype>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <exception>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "lbm_gb300.hpp"

namespace lbm {

template <typename M>
using Domain_ptr = std::unique_ptr<Domain<M>>;

namespace io {

// ------------------------------------------------------------------------------------------
// configuration.h
// ------------------------------------------------------------------------------------------
class Config {
    std::string _collision_model{"bgk"};
    std::string _input_file;
    std::string _output_dir{"vtk"};
    std::string _output_filename{"output"};
    std::string _scenario_xml;
    uint64_t _timesteps{0};
    uint64_t _timesteps_per_plot{0};
    double _tau{1.0};
    uint32_t _omp_threads{1};

    static std::string trim(const std::string& s)
    {
        size_t a = 0, b = s.size();
        while (a < b && std::isspace(static_cast<unsigned char>(s[a]))) ++a;
        while (b > a && std::isspace(static_cast<unsigned char>(s[b - 1]))) --b;
        return s.substr(a, b - a);
    }
    static bool known(const std::string& k)
    {
        static const char* names[] = {"collision-model", "tau", "timesteps", "timesteps-per-plot",
                                      "scenario-file", "omp-threads", "output-dir"};
        for (const char* n : names)
            if (k == n) return true;
        return false;
    }
    static void read_file(const std::string& path, std::map<std::string, std::string>& v)
    {
        std::ifstream in(path);
        if (!in) throw std::logic_error("can not read config file " + path);
        std::string line;
        while (std::getline(in, line)) {
            line = trim(line.substr(0, line.find('#')));
            if (line.empty()) continue;
            const size_t eq = line.find('=');
            if (eq == std::string::npos) throw std::logic_error("config line without '=': " + line);
            const std::string k = trim(line.substr(0, eq));
            if (!known(k)) throw std::logic_error("unrecognised option '" + k + "'");
            v.emplace(k, trim(line.substr(eq + 1)));  // the command line wins
        }
    }

public:
    auto collision_model() const -> decltype(_collision_model) { return _collision_model; }
    auto input_file() const -> decltype(_input_file) { return _input_file; }
    auto output_dir() const -> decltype(_output_dir) { return _output_dir; }
    auto output_filename() const -> decltype(_output_filename) { return _output_filename; }
    void set_output_filename(const std::string& filename) { _output_filename = filename; }
    auto timesteps() const -> decltype(_timesteps) { return _timesteps; }
    auto timesteps_per_plot() const -> decltype(_timesteps_per_plot) { return _timesteps_per_plot; }
    auto tau() const -> decltype(_tau) { return _tau; }
    auto omp_threads() const -> decltype(_omp_threads) { return _omp_threads; }
    auto scenario_xml() const -> decltype(_scenario_xml) { return _scenario_xml; }

    // Options: [file] -i/--input-file, -c/--collision-model, --tau, -t/--timesteps,
    // --timesteps-per-plot, --scenario-file, --omp-threads, --output-dir (--opt value or
    // --opt=value); unknown command-line options are ignored (allow_unregistered).
    Config(int argc, char** argv)
    {
        std::map<std::string, std::string> v;
        for (int i = 1; i < argc; ++i) {
            std::string a = argv[i], key, val;
            if (a == "-h" || a == "--help") {
                std::cout << "Usage: lbm_gb300_run [file] additional-options..." << std::endl;
                std::exit(1);
            }
            if (a.rfind("--", 0) == 0) {
                const size_t eq = a.find('=');
                key = a.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
                if (eq != std::string::npos) val = a.substr(eq + 1);
                else if (i + 1 < argc) val = argv[++i];
            } else if (a == "-i" || a == "-c" || a == "-t") {
                key = a == "-i" ? "input-file" : a == "-c" ? "collision-model" : "timesteps";
                if (i + 1 < argc) val = argv[++i];
            } else {
                _input_file = a;
                continue;
            }
            if (key == "input-file") _input_file = val;
            else if (known(key)) v[key] = val;
        }
        if (!_input_file.empty()) read_file(_input_file, v);
        for (const char* req : {"tau", "timesteps", "timesteps-per-plot", "scenario-file"})
            if (!v.count(req)) throw std::logic_error(std::string("the option '--") + req + "' is required but missing");
        try {
            if (v.count("collision-model")) _collision_model = v["collision-model"];
            _tau = std::stod(v["tau"]);
            _timesteps = std::stoull(v["timesteps"]);
            _timesteps_per_plot = std::stoull(v["timesteps-per-plot"]);
            _scenario_xml = v["scenario-file"];
            if (v.count("omp-threads")) _omp_threads = static_cast<uint32_t>(std::stoul(v["omp-threads"]));
            if (v.count("output-dir")) _output_dir = v["output-dir"];
        } catch (const std::invalid_argument&) {
            throw std::logic_error("invalid option value");
        }
        if (!(_timesteps > 0 && _tau > 0.5 && _tau < 2.0 && _omp_threads > 0 && _collision_model == "bgk"))
            throw std::logic_error("timesteps > 0, 0.5 < tau < 2, omp-threads > 0 and collision-model = bgk "
                                   "are required");
        // configuration.h:131-143: create the output directory or empty an existing one
        namespace fs = std::filesystem;
        const fs::path dir(_output_dir);
        if (!fs::exists(dir)) {
            std::cout << "Output directory \"" + _output_dir + "\" does not exist. Creating." << std::endl;
            fs::create_directories(dir);
        } else {
            for (const auto& f : fs::directory_iterator(dir))
                if (f.is_regular_file()) fs::remove(f.path());
        }
    }
};

inline std::ostream& operator<<(std::ostream& lhs, const Config& cfg)
{
    lhs << "Configuration:" << '\n'
        << "> Configuration file:     " << cfg.input_file() << '\n'
        << "> Output directory:       " << cfg.output_dir() << '\n'
        << "> Output filename:        " << cfg.output_filename() << '\n'
        << "> Collision model:        " << cfg.collision_model() << '\n'
        << "> Tau:                    " << cfg.tau() << '\n'
        << "> Timesteps:              " << cfg.timesteps() << '\n'
        << "> Timesteps per plot:     " << cfg.timesteps_per_plot() << '\n'
        << "> Scenario file:          " << cfg.scenario_xml();
    return lhs;
}

// ------------------------------------------------------------------------------------------
// a small XML reader: elements with attributes; text, comments and declarations are skipped
// ------------------------------------------------------------------------------------------
namespace xml {

struct Node {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<Node> children;

    const std::string* attr(const std::string& k) const
    {
        for (const auto& a : attrs)
            if (a.first == k) return &a.second;
        return nullptr;
    }
    const Node* child(const std::string& n) const
    {
        for (const auto& c : children)
            if (c.name == n) return &c;
        return nullptr;
    }
};

class Reader {
    const std::string& s;
    size_t i{0};

    [[noreturn]] void fail() const { throw std::runtime_error("xml"); }
    void skip_ws()
    {
        while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i;
    }
    bool starts(const char* t) const { return s.compare(i, std::strlen(t), t) == 0; }
    void skip_misc()  // whitespace, text, comments, <? ... ?>, <! ... >
    {
        for (;;) {
            while (i < s.size() && s[i] != '<') ++i;
            if (starts("<!--")) {
                const size_t e = s.find("-->", i + 4);
                if (e == std::string::npos) fail();
                i = e + 3;
            } else if (starts("<?") || (starts("<!") && !starts("<!--"))) {
                const size_t e = s.find('>', i);
                if (e == std::string::npos) fail();
                i = e + 1;
            } else {
                return;
            }
        }
    }
    std::string name()
    {
        const size_t a = i;
        while (i < s.size() && (std::isalnum(static_cast<unsigned char>(s[i])) || s[i] == '-' || s[i] == '_' ||
                                s[i] == ':' || s[i] == '.'))
            ++i;
        if (i == a) fail();
        return s.substr(a, i - a);
    }

public:
    explicit Reader(const std::string& text) : s(text) {}

    Node element()
    {
        skip_misc();
        if (i >= s.size() || s[i] != '<') fail();
        ++i;
        Node n;
        n.name = name();
        for (;;) {
            skip_ws();
            if (i >= s.size()) fail();
            if (s[i] == '/') {
                if (i + 1 >= s.size() || s[i + 1] != '>') fail();
                i += 2;
                return n;
            }
            if (s[i] == '>') {
                ++i;
                break;
            }
            std::string k = name();
            skip_ws();
            if (i >= s.size() || s[i] != '=') fail();
            ++i;
            skip_ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) fail();
            const char qch = s[i++];
            const size_t e = s.find(qch, i);
            if (e == std::string::npos) fail();
            n.attrs.emplace_back(k, s.substr(i, e - i));
            i = e + 1;
        }
        for (;;) {
            skip_misc();
            if (i >= s.size()) fail();
            if (starts("</")) {
                i += 2;
                if (name() != n.name) fail();
                skip_ws();
                if (i >= s.size() || s[i] != '>') fail();
                ++i;
                return n;
            }
            n.children.push_back(element());
        }
    }
};

}  // namespace xml

inline void check_attribute(const xml::Node& node, const std::string& name)
{
    if (!node.attr(name))
        throw std::logic_error("Missing attribute \"" + name + "\" for node \"" + node.name + "\"!");
}

// ------------------------------------------------------------------------------------------
// vtk.hpp:93-157
// ------------------------------------------------------------------------------------------
struct VtkPoints {
    size_t xl{0}, yl{0}, zl{0};
    double origin[3]{0, 0, 0}, spacing[3]{1, 1, 1};
    std::vector<std::uint8_t> fluid;  // x fastest
};

inline VtkPoints read_vtk_points(const std::string& filename)
{
    const std::string bad = "VTK file \"" + filename +
                            "\" does not exist or does not seem to be a valid structured grids file!";
    std::ifstream in(filename);
    if (!in) throw std::logic_error(bad);
    std::string line;
    for (int k = 0; k < 3; ++k)
        if (!std::getline(in, line)) throw std::logic_error(bad);  // version, title, ASCII
    if (line.find("ASCII") == std::string::npos) throw std::logic_error(bad + " (only ASCII files)");
    VtkPoints p;
    std::string tok;
    bool sp = false;
    size_t npts = 0;
    while (in >> tok) {
        if (tok == "DATASET") {
            in >> tok;
            sp = tok == "STRUCTURED_POINTS";
        } else if (tok == "DIMENSIONS") {
            in >> p.xl >> p.yl >> p.zl;
        } else if (tok == "ORIGIN") {
            in >> p.origin[0] >> p.origin[1] >> p.origin[2];
        } else if (tok == "SPACING" || tok == "ASPECT_RATIO") {
            in >> p.spacing[0] >> p.spacing[1] >> p.spacing[2];
        } else if (tok == "POINT_DATA") {
            in >> npts;
            break;
        }
    }
    if (!sp || p.xl * p.yl * p.zl == 0 || npts != p.xl * p.yl * p.zl) throw std::logic_error(bad);
    in >> tok;  // SCALARS name type [ncomp]
    if (tok == "SCALARS") {
        std::string rest;
        std::getline(in, rest);
        in >> tok;
        if (tok == "LOOKUP_TABLE") in >> tok;
        else throw std::logic_error(bad);
    } else {
        throw std::logic_error("Point data is null!");
    }
    p.fluid.resize(npts);
    for (size_t k = 0; k < npts; ++k) {
        double v;
        if (!(in >> v)) throw std::logic_error(bad + " (too few values)");
        p.fluid[k] = v != 0.0;
    }
    return p;
}

// A domain sized, placed and spaced by the file; points with value 0 are solid cells of the
// handler type solid_collision_model (the reference instantiates NoSlipBoundary here; this build
// binds them to its no-slip handler).
template <typename lattice_model, typename solid_collision_model = NoSlipBoundary<lattice_model>>
Domain_ptr<lattice_model> read_vtk_point_file(const std::string& filename,
                                              FluidCollision<lattice_model>& fluid_collision_model,
                                              int precision = LBM_FP64)
{
    const VtkPoints p = read_vtk_points(filename);
    auto domain = std::make_unique<Domain<lattice_model>>(
        p.xl, p.yl, p.zl, fluid_collision_model, p.origin[0], p.origin[1], p.origin[2], p.spacing[0],
        p.spacing[1], p.spacing[2], precision);
    std::vector<std::uint8_t> solid(p.fluid.size());
    for (size_t k = 0; k < solid.size(); ++k) solid[k] = p.fluid[k] ? 0 : 1;
    domain->set_solid_mask(solid);
    return domain;
}

// ------------------------------------------------------------------------------------------
// scenario.h:29-188
// ------------------------------------------------------------------------------------------
template <typename lattice_model>
NonFluidCollision<lattice_model>& parse_condition(const xml::Node& boundary, Domain<lattice_model>& domain)
{
    using BF = BoundaryKeeper<lattice_model>;
    check_attribute(boundary, "condition");
    const std::string condition = *boundary.attr("condition");
    auto num = [&](const char* k) { return std::stod(*boundary.attr(k)); };
    if (condition == "noslip") return BF::template get_collision<NoSlipBoundary<lattice_model>>(domain);
    if (condition == "movingwall" || condition == "inflow") {
        check_attribute(boundary, "vx");
        check_attribute(boundary, "vy");
        check_attribute(boundary, "vz");
        const double_array<lattice_model::D> v = {num("vx"), num("vy"), num("vz")};
        if (condition == "movingwall")
            return BF::template get_collision<MovingWallBoundary<lattice_model>>(domain, v);
        const double rho_ref = boundary.attr("rho-ref") ? num("rho-ref") : 1.0;
        return BF::template get_collision<InflowBoundary<lattice_model>>(domain, v, rho_ref);
    }
    if (condition == "freeslip") return BF::template get_collision<FreeSlipBoundary<lattice_model>>(domain);
    if (condition == "outflow") {
        const double rho_ref = boundary.attr("rho-ref") ? num("rho-ref") : 1.0;
        return BF::template get_collision<OutflowBoundary<lattice_model>>(domain, rho_ref);
    }
    if (condition == "pressure") {
        check_attribute(boundary, "rho-in");
        return BF::template get_collision<PressureBoundary<lattice_model>>(domain, num("rho-in"));
    }
    throw std::logic_error(condition + " boundary condition not supported!");
}

template <typename lattice_model>
void parse_boundary(const xml::Node& boundary, Domain<lattice_model>& domain)
{
    check_attribute(boundary, "extent");
    const std::string extent = *boundary.attr("extent");
    auto& condition = parse_condition<lattice_model>(boundary, domain);
    const size_t xl = domain.xlength(), yl = domain.ylength(), zl = domain.zlength();
    if (extent == "z0") domain.setBoundaryCondition(condition, 0, xl + 1, 0, yl + 1, 0, 0);
    else if (extent == "zmax") domain.setBoundaryCondition(condition, 0, xl + 1, 0, yl + 1, zl + 1, zl + 1);
    else if (extent == "x0") domain.setBoundaryCondition(condition, 0, 0, 0, yl + 1, 0, zl + 1);
    else if (extent == "xmax") domain.setBoundaryCondition(condition, xl + 1, xl + 1, 0, yl + 1, 0, zl + 1);
    else if (extent == "y0") domain.setBoundaryCondition(condition, 0, xl + 1, 0, 0, 0, zl + 1);
    else if (extent == "ymax") domain.setBoundaryCondition(condition, 0, xl + 1, yl + 1, yl + 1, 0, zl + 1);
    else {
        std::vector<std::uint64_t> ex;
        std::istringstream ss(extent);
        std::string t;
        while (ss >> t) {
            try {
                ex.push_back(std::stoull(t));
            } catch (const std::exception&) {
                throw std::logic_error("Extent \"" + extent + "\" is not complete! Must be six values!");
            }
        }
        if (ex.size() < 6) throw std::logic_error("Extent \"" + extent + "\" is not complete! Must be six values!");
        domain.setBoundaryCondition(condition, ex[0], ex[1], ex[2], ex[3], ex[4], ex[5]);
    }
}

// The vtk-file of a domain node is looked up relative to the working directory (as the
// reference does) and, failing that, relative to the scenario file's directory.
template <typename lattice_model>
Domain_ptr<lattice_model> parse_scenario_file(const std::string& filename, Config& cfg,
                                              FluidCollision<lattice_model>& collision,
                                              int precision = LBM_FP64)
{
    std::ifstream in(filename);
    std::stringstream buf;
    if (in) buf << in.rdbuf();
    xml::Node doc;
    try {
        if (!in) throw std::runtime_error("xml");
        doc = xml::Reader(buf.str()).element();
    } catch (const std::runtime_error&) {
        throw std::logic_error("XML file \"" + filename + "\" could not be read properly!");
    }
    const xml::Node* scenario = doc.name == "scenario" ? &doc : doc.child("scenario");
    if (!scenario) throw std::logic_error("Scenario node missing!");
    if (!scenario->attr("name")) throw std::logic_error("Scenario name is missing!");
    const std::string scenario_name = *scenario->attr("name");
    std::cout << "Reading scenario: \"" << scenario_name << "\"..." << std::endl;
    cfg.set_output_filename(scenario_name);
    const xml::Node* xml_domain = scenario->child("domain");
    if (!xml_domain) throw std::logic_error("Domain node is missing!");
    Domain_ptr<lattice_model> domain;
    if (const std::string* vtk = xml_domain->attr("vtk-file")) {
        namespace fs = std::filesystem;
        fs::path path(*vtk);
        if (!fs::exists(path) && fs::exists(fs::path(filename).parent_path() / path))
            path = fs::path(filename).parent_path() / path;
        domain = read_vtk_point_file<lattice_model>(path.string(), collision, precision);
    } else if (xml_domain->attr("xl") && xml_domain->attr("yl") && xml_domain->attr("zl")) {
        const long xl = std::stol(*xml_domain->attr("xl")), yl = std::stol(*xml_domain->attr("yl")),
                   zl = std::stol(*xml_domain->attr("zl"));
        if (xl <= 0 || yl <= 0 || zl <= 0) throw std::logic_error("domain lengths must be positive");
        domain = std::make_unique<Domain<lattice_model>>(xl, yl, zl, collision, 0, 0, 0, 1, 1, 1, precision);
    } else {
        throw std::logic_error("Neither vtk-file nor xl/yl/zl attribute provided to domain node!");
    }
    for (const auto& c : xml_domain->children)
        if (c.name == "boundary") parse_boundary(c, *domain);
    return domain;
}

// ------------------------------------------------------------------------------------------
// vtk.hpp:13-89: VTS output
// ------------------------------------------------------------------------------------------
namespace detail_vts {
inline std::string base64_block(const void* data, uint32_t nbytes)
{
    static const char* tab = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::vector<unsigned char> raw(4 + static_cast<size_t>(nbytes));
    std::memcpy(raw.data(), &nbytes, 4);  // little-endian hosts (x86-64, AArch64)
    std::memcpy(raw.data() + 4, data, nbytes);
    std::string out;
    out.reserve((raw.size() + 2) / 3 * 4);
    size_t k = 0;
    for (; k + 2 < raw.size(); k += 3) {
        const uint32_t v = (raw[k] << 16) | (raw[k + 1] << 8) | raw[k + 2];
        out += tab[v >> 18];
        out += tab[(v >> 12) & 63];
        out += tab[(v >> 6) & 63];
        out += tab[v & 63];
    }
    if (k < raw.size()) {
        const uint32_t v = (raw[k] << 16) | (k + 1 < raw.size() ? raw[k + 1] << 8 : 0);
        out += tab[v >> 18];
        out += tab[(v >> 12) & 63];
        out += k + 1 < raw.size() ? tab[(v >> 6) & 63] : '=';
        out += '=';
    }
    return out;
}
}  // namespace detail_vts

// One output file's data: the moments of the interior cells at one step, read from the device,
// and what the file names and places.
struct VtsSnapshot {
    size_t xl = 0, yl = 0, zl = 0;
    double xo = 0, yo = 0, zo = 0, xs = 1, ys = 1, zs = 1;
    std::vector<double> rho, u;
    std::string path;
};

template <typename lattice_model>
VtsSnapshot vts_snapshot(const Domain<lattice_model>& domain, const std::string& output_dir,
                         const std::string& output_filename, uint64_t t)
{
    VtsSnapshot s;
    s.xl = domain.xlength(), s.yl = domain.ylength(), s.zl = domain.zlength();
    s.xo = domain.xorigin(), s.yo = domain.yorigin(), s.zo = domain.zorigin();
    s.xs = domain.xspacing(), s.ys = domain.yspacing(), s.zs = domain.zspacing();
    domain.moments(s.rho, s.u);
    std::ostringstream name;
    name << output_dir << "/" << output_filename << "." << t << ".vts";
    s.path = name.str();
    return s;
}

// The file of a snapshot: point data "Velocity" (3 x Float64) and "Density" (Float64) of the
// interior cells, x fastest, at points (xs*x + xo - 1, ys*y + yo - 1, zs*z + zo - 1), x = 1..xl
// etc. (Float32).
inline void write_vts(const VtsSnapshot& s)
{
    const size_t xl = s.xl, yl = s.yl, zl = s.zl;
    std::vector<float> pts(3 * xl * yl * zl);
    size_t k = 0;
    for (size_t z = 1; z <= zl; ++z)
        for (size_t y = 1; y <= yl; ++y)
            for (size_t x = 1; x <= xl; ++x) {
                pts[k++] = static_cast<float>(s.xs * x + s.xo - 1);
                pts[k++] = static_cast<float>(s.ys * y + s.yo - 1);
                pts[k++] = static_cast<float>(s.zs * z + s.zo - 1);
            }
    std::ofstream file(s.path, std::ios::trunc | std::ios::binary);
    if (!file) throw std::logic_error("Failed to open file " + s.path);
    const std::string ext = "0 " + std::to_string(xl - 1) + " 0 " + std::to_string(yl - 1) + " 0 " +
                            std::to_string(zl - 1);
    using detail_vts::base64_block;
    file << "<?xml version=\"1.0\"?>\n"
         << "<VTKFile type=\"StructuredGrid\" version=\"0.1\" byte_order=\"LittleEndian\" header_type=\"UInt32\">\n"
         << "  <StructuredGrid WholeExtent=\"" << ext << "\">\n"
         << "    <Piece Extent=\"" << ext << "\">\n"
         << "      <PointData Scalars=\"Density\" Vectors=\"Velocity\">\n"
         << "        <DataArray type=\"Float64\" Name=\"Velocity\" NumberOfComponents=\"3\" format=\"binary\">\n"
         << base64_block(s.u.data(), static_cast<uint32_t>(s.u.size() * sizeof(double))) << "\n"
         << "        </DataArray>\n"
         << "        <DataArray type=\"Float64\" Name=\"Density\" format=\"binary\">\n"
         << base64_block(s.rho.data(), static_cast<uint32_t>(s.rho.size() * sizeof(double))) << "\n"
         << "        </DataArray>\n"
         << "      </PointData>\n"
         << "      <CellData></CellData>\n"
         << "      <Points>\n"
         << "        <DataArray type=\"Float32\" NumberOfComponents=\"3\" format=\"binary\">\n"
         << base64_block(pts.data(), static_cast<uint32_t>(pts.size() * sizeof(float))) << "\n"
         << "        </DataArray>\n"
         << "      </Points>\n"
         << "    </Piece>\n"
         << "  </StructuredGrid>\n"
         << "</VTKFile>\n";
    if (!file) throw std::logic_error("Failed to write file " + s.path);
}

// vtk.hpp:42-89: <output_dir>/<output_filename>.<t>.vts from the device moments, written on the
// caller's thread.
template <typename lattice_model>
void write_vtk_file(const Domain<lattice_model>& domain, const std::string& output_dir,
                    const std::string& output_filename, uint64_t t)
{
    write_vts(vts_snapshot(domain, output_dir, output_filename, t));
}

// Extension: the reference writes every file on the time loop's thread (main.cpp:56-57), so the
// solver waits while the moments are encoded and written. submit() reads the moments from the
// device (one synchronising read-back) and hands the file to a background thread; the loop then
// goes on launching steps while the file is written. At most `depth` snapshots wait in host memory
// (submit blocks beyond that). A failed write is rethrown by the next submit() or by finish();
// the destructor finishes the queue and drops any error.
class VtkWriter {
public:
    explicit VtkWriter(size_t depth = 2) : depth_(depth ? depth : 1), worker_([this] { run(); }) {}
    VtkWriter(const VtkWriter&) = delete;
    VtkWriter& operator=(const VtkWriter&) = delete;
    ~VtkWriter()
    {
        try {
            finish();
        } catch (...) {
        }
        {
            std::lock_guard<std::mutex> lock(m_);
            stop_ = true;
        }
        cv_.notify_all();
        worker_.join();
    }

    template <typename lattice_model>
    void submit(const Domain<lattice_model>& domain, const std::string& output_dir,
                const std::string& output_filename, uint64_t t)
    {
        VtsSnapshot s = vts_snapshot(domain, output_dir, output_filename, t);
        std::unique_lock<std::mutex> lock(m_);
        rethrow_locked();
        cv_.wait(lock, [this] { return queue_.size() < depth_; });
        queue_.push_back(std::move(s));
        cv_.notify_all();
    }

    // Waits until every submitted file is written; rethrows the first failure.
    void finish()
    {
        std::unique_lock<std::mutex> lock(m_);
        cv_.wait(lock, [this] { return queue_.empty() && !busy_; });
        rethrow_locked();
    }

private:
    void rethrow_locked()
    {
        if (error_) {
            std::exception_ptr e = error_;
            error_ = nullptr;
            std::rethrow_exception(e);
        }
    }
    void run()
    {
        std::unique_lock<std::mutex> lock(m_);
        for (;;) {
            cv_.wait(lock, [this] { return stop_ || !queue_.empty(); });
            if (queue_.empty()) return;  // stop requested and nothing left
            VtsSnapshot s = std::move(queue_.front());
            queue_.pop_front();
            busy_ = true;
            lock.unlock();
            try {
                write_vts(s);
            } catch (...) {
                lock.lock();
                if (!error_) error_ = std::current_exception();
                lock.unlock();
            }
            lock.lock();
            busy_ = false;
            cv_.notify_all();
        }
    }

    size_t depth_;
    std::mutex m_;
    std::condition_variable cv_;
    std::deque<VtsSnapshot> queue_;
    bool busy_ = false;
    bool stop_ = false;
    std::exception_ptr error_;
    std::thread worker_;
};

}  // namespace io
}  // namespace lbm
