// ratpoints-compatible command line, output formatter and program entry.
//
// Restates the reference's CLI contract so its harnesses and callers can run
// this binary unchanged:
//   - parse_command_line / OptionParser (src/command_line.cpp:113-366);
//   - OutputFormatter (src/output_formatter.cpp:7-105);
//   - main, --help, --list-devices and the -v metrics line (src/main.cpp:14-85).
// Two extensions: --sieve-plan reference|fast selects the sieve plan (default
// fast; reference reproduces the reference's modular survivor set and counts),
// and --host-verify-only sends every modular survivor to the host's exact check
// (by default a device kernel first drops those that cannot be points).
#include "cli.hpp"

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "search.hpp"

namespace rpg {

namespace {

constexpr int kMaximumDegree = 100;
constexpr long long kMaximumHeight = (std::numeric_limits<long long>::max() - 32) / 2;
constexpr char kUsage[] = "Usage: ratpoints_gpu 'c0 c1 ... cn' HEIGHT [OPTIONS]";

struct OutputOptions {
    bool print_points = true;
    bool print_y = true;
    std::string format, before, between, after;
};

struct ProgramOptions {
    SearchOptions search;
    OutputOptions output;
    bool quiet = false, verbose = false, stop_after_first = false;
};

long long parse_positive(const char *text, const char *name) {
    errno = 0;
    char *end = nullptr;
    long long value = std::strtoll(text, &end, 10);
    if (errno == ERANGE || end == text || *end || value < 1)
        throw std::invalid_argument(std::string(name) + " must be positive");
    return value;
}

int parse_positive_int(const char *text, const char *name) {
    long long value = parse_positive(text, name);
    if (value > std::numeric_limits<int>::max())
        throw std::invalid_argument(std::string(name) + " exceeds GPU limit");
    return int(value);
}

Rational real_or_throw(const char *text, const char *name) {
    Rational r;
    std::string error;
    if (!parse_real(text, name, r, error)) throw std::invalid_argument(error);
    return r;
}

bool is_integer(const std::string &text) {
    std::size_t i = !text.empty() && (text[0] == '-' || text[0] == '+');
    if (i == text.size()) return false;
    for (; i < text.size(); ++i)
        if (text[i] < '0' || text[i] > '9') return false;
    return true;
}

bool is_zero(const std::string &text) {
    std::size_t i = !text.empty() && (text[0] == '-' || text[0] == '+');
    for (; i < text.size(); ++i)
        if (text[i] != '0') return false;
    return true;
}

std::vector<std::string> split_coefficients(const char *text) {
    std::istringstream stream(text);
    std::vector<std::string> out;
    for (std::string token; stream >> token;) {
        if (!token.empty() && token.front() == '+') token.erase(0, 1);
        out.push_back(token);
    }
    return out;
}

void validate_coefficients(const std::vector<std::string> &c) {
    if (c.size() < 2 || c.size() > std::size_t(kMaximumDegree + 1))
        throw std::invalid_argument("supported polynomial degrees are 1 through 100");
    for (const auto &x : c)
        if (!is_integer(x)) throw std::invalid_argument("coefficients must be decimal integers");
    if (is_zero(c.back())) throw std::invalid_argument("leading coefficient must be nonzero");
}

class OptionParser {
public:
    OptionParser(int argc, char **argv, ProgramOptions &result)
        : argc_(argc), argv_(argv), result_(result) {}

    void parse() {
        while (index_ < argc_) {
            std::string option(argv_[index_++]);
            if (search_option(option) || output_option(option) || runtime_option(option)) continue;
            throw std::invalid_argument("unsupported ratpoints option: " + option);
        }
        if (has_pending_) {
            SearchInterval iv;
            iv.lower = pending_;
            iv.upper_infinite = true;
            result_.search.intervals.push_back(iv);
        }
    }

private:
    const char *argument(const std::string &option) {
        if (index_ >= argc_) throw std::invalid_argument(option + " requires an argument");
        return argv_[index_++];
    }

    bool search_option(const std::string &o) {
        if (o == "-dl") {
            result_.search.first = parse_positive_int(argument(o), "lower denominator");
        } else if (o == "-du") {
            result_.search.last = parse_positive_int(argument(o), "upper denominator");
        } else if (o == "-l") {
            if (has_pending_) throw std::invalid_argument("interval lower bound without upper bound");
            pending_ = real_or_throw(argument(o), "interval lower bound");
            has_pending_ = true;
        } else if (o == "-u") {
            Rational upper = real_or_throw(argument(o), "interval upper bound");
            if (has_pending_ && Rational::compare(pending_, upper) > 0)
                throw std::invalid_argument("interval lower bound exceeds upper bound");
            auto &ivs = result_.search.intervals;
            if (!ivs.empty() && (!has_pending_ || ivs.back().upper_infinite ||
                                 Rational::compare(pending_, ivs.back().upper) < 0))
                throw std::invalid_argument("search intervals must be ordered");
            SearchInterval iv;
            iv.lower = pending_;
            iv.upper = upper;
            iv.lower_infinite = !has_pending_;
            ivs.push_back(iv);
            has_pending_ = false;
        } else if (o == "-i") {
            result_.search.include_infinity = false;
        } else if (o == "-I") {
            result_.search.include_infinity = true;
        } else {
            return false;
        }
        return true;
    }

    bool output_option(const std::string &o) {
        auto &out = result_.output;
        if (o == "-y") out.print_y = false;
        else if (o == "-Y") out.print_y = true;
        else if (o == "-z") out.print_points = false;
        else if (o == "-Z") out.print_points = true;
        else if (o == "-f") out.format = argument(o);
        else if (o == "-fs") out.before = argument(o);
        else if (o == "-fm") out.between = argument(o);
        else if (o == "-fe") out.after = argument(o);
        else return false;
        return true;
    }

    bool runtime_option(const std::string &o) {
        auto &s = result_.search;
        if (o == "--devices") {
            s.devices = parse_device_selection(argument(o));
        } else if (o == "--batch-size") {
            s.batch_size = parse_positive_int(argument(o), "denominator batch size");
            if (s.batch_size > (1 << 16))
                throw std::invalid_argument("--batch-size must not exceed 65536");
        } else if (o == "--square-denominators") {
            s.square = true;
        } else if (o == "--sieve-plan") {
            std::string v = argument(o);
            if (v == "reference") s.plan = PlanKind::reference;
            else if (v == "fast") s.plan = PlanKind::fast;
            else throw std::invalid_argument("--sieve-plan must be reference or fast");
        } else if (o == "--host-verify-only") {
            s.device_preverify = false;
        } else if (o == "-q") {
            result_.quiet = true;
        } else if (o == "-v") {
            result_.verbose = true;
        } else if (o == "-1") {
            result_.stop_after_first = true;
        } else if (o == "-s" || o == "-k" || o == "-K" || o == "-j" || o == "-J") {
            // Accepted with no effect, as in the reference (command_line.cpp:252-254).
        } else {
            return false;
        }
        return true;
    }

    int argc_;
    char **argv_;
    ProgramOptions &result_;
    int index_ = 3;
    Rational pending_;
    bool has_pending_ = false;
};

ProgramOptions parse_command_line(int argc, char **argv) {
    if (argc < 3) throw std::invalid_argument(kUsage);
    ProgramOptions r;
    r.search.coefficients = split_coefficients(argv[1]);
    r.search.numerator_bound = parse_positive(argv[2], "maximum height");
    if (r.search.numerator_bound > kMaximumHeight)
        throw std::invalid_argument("maximum height exceeds safe GPU limit");
    r.search.last = r.search.numerator_bound > std::numeric_limits<int>::max()
                        ? std::numeric_limits<int>::max()
                        : r.search.numerator_bound;
    OptionParser(argc, argv, r).parse();
    if (r.search.last > r.search.numerator_bound) r.search.last = r.search.numerator_bound;
    if (r.search.square && r.search.last > 46340) r.search.last = 46340;
    if (r.search.first > r.search.last) throw std::invalid_argument("empty denominator range");
    validate_coefficients(r.search.coefficients);
    return r;
}

class OutputFormatter {
public:
    explicit OutputFormatter(const OutputOptions &o)
        : print_points_(o.print_points), print_y_(o.print_y),
          format_(decode(o.format.empty() ? (o.print_y ? "(%x : %y : %z)\\n" : "(%x : %z)\\n")
                                          : o.format)),
          before_(decode(o.before)), between_(decode(o.between)), after_(decode(o.after)) {
        if (print_points_) write(before_);
    }

    void point_pair(const PointPair &p, bool include_conjugate) {
        write_point(p.numerator, p.ordinate, p.denominator);
        if (include_conjugate && print_y_ && p.ordinate != "0")
            write_point(p.numerator, "-" + p.ordinate, p.denominator);
    }

    void finish() {
        if (finished_) return;
        write(after_);
        if (std::fflush(stdout) == EOF) throw std::runtime_error("failed to flush standard output");
        finished_ = true;
    }

private:
    static constexpr char kEscapedPercent = '\x01';

    static std::string decode(const std::string &in) {
        std::string out;
        for (std::size_t i = 0; i < in.size(); ++i) {
            if (in[i] != '\\' || i + 1 == in.size()) {
                out.push_back(in[i]);
                continue;
            }
            char e = in[++i];
            if (e == 'n') out.push_back('\n');
            else if (e == 't') out.push_back('\t');
            else if (e == '%') out.push_back(kEscapedPercent);
            else {
                out.push_back('\\');
                out.push_back(e);
            }
        }
        return out;
    }

    static void write(const std::string &text) {
        if (std::fputs(text.c_str(), stdout) == EOF)
            throw std::runtime_error("failed to write standard output");
    }

    void write_point(long long numerator, const std::string &ordinate, long long denominator) {
        if (!print_points_) return;
        if (emitted_) write(between_);
        std::string s;
        for (std::size_t i = 0; i < format_.size(); ++i) {
            if (format_[i] != '%' || i + 1 == format_.size()) {
                s.push_back(format_[i]);
                continue;
            }
            char m = format_[i + 1];
            if (m == 'x') s += std::to_string(numerator);
            else if (m == 'y' && print_y_) s += ordinate;
            else if (m == 'z') s += std::to_string(denominator);
            else {
                s.push_back('%');
                s.push_back(m);
            }
            ++i;
        }
        for (char &c : s)
            if (c == kEscapedPercent) c = '%';
        write(s);
        emitted_ = true;
    }

    bool print_points_, print_y_;
    std::string format_, before_, between_, after_;
    bool emitted_ = false, finished_ = false;
};

void print_help(std::FILE *stream) {
    static const char text[] =
        "Usage: ratpoints_gpu 'c0 c1 ... cn' HEIGHT [OPTIONS]\n"
        "\n"
        "Search y^2 = c0 + c1 x + ... + cn x^n for x = a/b with |a| <= HEIGHT.\n"
        "\n"
        "Device options:\n"
        "  --devices all|0,1,...  choose CUDA-visible GPUs; the first one runs the search\n"
        "  --batch-size N         denominators per batch, 1..65536 (default 65536)\n"
        "  --square-denominators  treat -dl/-du as bounds on k and search d = k^2\n"
        "  --sieve-plan P         reference or fast (default fast); same points either way\n"
        "  --host-verify-only     check every modular survivor on the host (no device pre-verification)\n"
        "  --list-devices         print the visible GPUs and exit\n"
        "\n"
        "Search and output options:\n"
        "  -dl B, -du B   lower and upper denominator bounds\n"
        "  -l L, -u U     start and end a closed interval for x (repeatable)\n"
        "  -1             stop after the first point\n"
        "  -i, -I         leave out or include points at infinity\n"
        "  -y, -Y         leave out or include ordinates\n"
        "  -z, -Z         leave out or include point lines\n"
        "  -q             no timing output\n"
        "  -v             timing and survivor metrics on standard error\n"
        "  -f FORMAT      point format with %x, %y, %z\n"
        "  -fs, -fm, -fe  text before, between and after the points\n"
        "  -s, -k, -K, -j, -J  accepted, no effect\n"
        "  --help         this text\n";
    if (std::fputs(text, stream) == EOF) throw std::runtime_error("failed to write help output");
}

void print_device(std::FILE *stream, const GpuDevice &d) {
    std::fprintf(stream, "device=%d name=\"%s\" compute=%d.%d sm=%d memory_mib=%llu pci=%s\n", d.id,
                 d.name.c_str(), d.major, d.minor, d.multiprocessors,
                 d.memory_bytes / (1024ULL * 1024ULL), d.pci_bus_id.c_str());
}

void print_metrics(const SearchMetrics &m) {
    std::fprintf(stderr,
                 "wall_ms=%.3f devices=%zu denominators=%llu basis_ms=%.3f sieve_ms=%.3f words=%llu "
                 "initial_mask_gbs=%.3f survivors=%llu exact_survivors=%llu plan_ms=%.3f "
                 "workspace_ms=%.3f basis_wall_ms=%.3f survivor_setup_ms=%.3f "
                 "verification_ms=%.3f sieve_wall_ms=%.3f\n",
                 m.wall_ms, m.devices.size(), m.denominator_count, m.basis_ms, m.sieve_ms,
                 m.word_count, m.initial_mask_gbs(), m.modular_survivors, m.exact_survivors,
                 m.plan_ms, m.workspace_ms, m.basis_wall_ms, m.survivor_setup_ms,
                 m.verification_ms, m.sieve_wall_ms);
    for (const auto &e : m.devices) {
        print_device(stderr, e.device);
        std::fprintf(stderr, "gpu=%d denominators=%llu batches=%llu basis_ms=%.3f sieve_ms=%.3f\n",
                     e.device.id, e.denominator_count, e.batches, e.basis_ms, e.sieve_ms);
    }
}

}  // namespace

int run_cli(int argc, char **argv) {
    try {
        if (argc == 1) {
            print_help(stderr);
            return 1;
        }
        if (argc == 2 && std::string(argv[1]) == "--help") {
            print_help(stdout);
            return 0;
        }
        if (argc == 2 && std::string(argv[1]) == "--list-devices") {
            for (const auto &d : available_gpu_devices()) print_device(stdout, d);
            return std::fflush(stdout) == EOF ? 1 : 0;
        }
        ProgramOptions options = parse_command_line(argc, argv);
        PointSearch search(options.search);
        OutputFormatter output(options.output);
        const bool stop = options.stop_after_first;
        SearchMetrics metrics = search.run([&](const PointPair &p) {
            output.point_pair(p, !stop);
            return !stop;
        });
        output.finish();
        if (std::getenv("RATPOINTS_GPU_BENCHMARK") != nullptr || (options.verbose && !options.quiet))
            print_metrics(metrics);
        return 0;
    } catch (const std::exception &error) {
        std::fflush(stdout);
        std::fprintf(stderr, "%s\n", error.what());
        return 1;
    }
}

}  // namespace rpg
