// boids_cli.h -- host side of the boidsim / boidsim_grid command lines.
//
// The reference builds its CLI (src/main.cpp, src/args.cpp) on Boost
// program_options and property_tree; this is a Boost-free restatement of the
// same surface over the C ABI of include/boids.h:
//   * options and their precedence (src/args.cpp:21-153): -s/--setting .ini
//     first, then the command-line values on top;
//   * the .ini reader with property_tree's read_ini rules and its
//     get_optional<T> conversions (src/args.cpp:78-128);
//   * the .ptcl v0.2 writer (header src/dtype.h:19-35 written by
//     src/main.cpp:60-74; one frame per step written before the update,
//     src/main.cpp:187-291), fed by a double-buffered, asynchronous
//     device-to-host frame pipeline instead of per-boid getter calls.
#ifndef BOIDS_CLI_H
#define BOIDS_CLI_H

#include <cstdint>
#include <map>
#include <optional>
#include <string>

namespace boidscli {

// property_tree's ini tree: section -> key -> value (keys outside a section
// live under the empty section name).  read() throws std::runtime_error
// with read_ini's message, "<file>(<line>): <what>".
struct IniFile {
    std::map<std::string, std::map<std::string, std::string>> sections;
    static IniFile read(const std::string &path);
    static IniFile parse(const std::string &text, const std::string &name);
    // "Section.KEY" lookup; null when absent.
    const std::string *find(const std::string &dotted) const;
};

// Conversions with the acceptance rules of the reference's two parsers.
// ini values (property_tree stream_translator over std::istream >>) and
// command-line values (boost::lexical_cast) accept the same plain decimal
// forms; the command line also takes inf/nan for doubles.  Unsigned values
// may carry a sign and wrap modulo 2^32, as both of the reference's parsers
// do for "-1".
bool parse_unsigned(const std::string &s, unsigned &out);
bool parse_int(const std::string &s, int &out);
bool parse_double(const std::string &s, double &out, bool allow_special);

// The values of class Args (src/args.h:7-33).  Parameters the reference
// leaves indeterminate when neither the .ini nor the command line sets them
// are empty optionals here and rejected before the run.
struct Args {
    std::string setting_filename;
    std::string output_filename;
    std::string velocity_output_filename;
    bool is_parallel_output = false;   // accepted and ignored, as in a non-MPI build
    bool is_force_data_output = false;
    bool output_given = false;
    bool initialization_given = false;
    std::optional<unsigned> time_step;
    std::optional<unsigned> population;
    std::optional<double> field_size;
    std::optional<double> separation_sight_distance, separation_sight_angle, separation_force_coefficient;
    std::optional<double> alignment_sight_distance, alignment_sight_angle, alignment_force_coefficient;
    std::optional<double> cohesion_sight_distance, cohesion_sight_angle, cohesion_force_coefficient;
    std::optional<double> velocity_max, velocity_min;
    std::optional<std::string> initialization;
    std::optional<int> random_seed;
    // options of this build only (no reference counterpart)
    unsigned output_interval = 1;  // write every k-th frame
    int device = 0;                // CUDA device ordinal
    bool quiet = false;            // no per-step progress lines
    bool print_config = false;     // print the resolved values, do not run
};

// key=value lines of the resolved Args (doubles with 17 significant
// digits, "unset" for an empty optional).
std::string format_config(const Args &a);

enum ParseResult { PARSE_OK = 0, PARSE_HELP = 1, PARSE_ERROR = -1 };

// Parses argv like Args::Args (src/args.cpp:17-154).  On PARSE_ERROR, err
// holds the message the reference prints before exit(-1).
ParseResult parse_args(int argc, const char *const *argv, Args &out, std::string &err);

// Text for --help.
std::string usage(const char *prog);

// Applies an .ini tree to args (src/args.cpp:78-128); command-line values
// given afterwards override these.
void apply_ini(const IniFile &ini, Args &args);

// The simulation run of src/main.cpp:77-303 for one engine
// (BOIDS_ENGINE_ALLPAIRS for boidsim, BOIDS_ENGINE_GRID for boidsim_grid).
// Returns the process exit status.
int run(const Args &args, int engine, const char *prog);

// 50-byte data_file_header_v02 as src/main.cpp:60-74 fills it.
struct PtclHeader {
    uint32_t n, steps, t0;
    float field;
};
void encode_header(const PtclHeader &h, unsigned char out[50]);

}  // namespace boidscli

#endif
