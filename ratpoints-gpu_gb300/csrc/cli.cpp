// The ratpoints_gpu command line: argument grammar, output rendering and the
// program's top-level flow.
//
// The observable contract is the reference's and is kept byte for byte: the
// option names and their arguments, the defaults and clamps, every error
// message and the order in which errors are detected (src/command_line.cpp:
// 336-366), the stdout bytes of a search (src/output_formatter.cpp), the -v
// metrics line and the --list-devices line (src/main.cpp:14-43), and the exit
// codes (src/main.cpp:48-85).  The code is this project's own: options are
// looked up in one table and applied by a single dispatcher, and the point
// format is compiled once into a list of pieces that is rendered per point.
// Two extensions: --sieve-plan reference|fast selects the sieve plan (default
// fast; reference reproduces the reference's modular survivor set and counts),
// and --host-verify-only sends every modular survivor to the host's exact check
// (by default a device kernel first drops those that cannot be points).
#include "cli.hpp"

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "point_format.hpp"
#include "search.hpp"

namespace rpg {

namespace {

constexpr std::size_t kMostCoefficients = 101;  // degree 100
constexpr long long kHeightCeiling = (std::numeric_limits<long long>::max() - 32) / 2;
constexpr int kSquareDenominatorCeiling = 46340;  // floor(sqrt(2^31 - 1))
constexpr int kLargestBatch = 1 << 16;

[[noreturn]] void usage_error(const std::string &message) { throw std::invalid_argument(message); }

// ---------------------------------------------------------------------------
// Settings the command line produces

struct Invocation {
    SearchOptions search;
    RenderSettings render;
    bool quiet = false;
    bool verbose = false;
    bool first_point_only = false;
};

// ---------------------------------------------------------------------------
// Scalar arguments

// A positive decimal count as strtoll reads it (leading blanks and a sign are
// allowed, nothing may follow); anything else is "<what> must be positive".
long long positive_count(const char *text, const std::string &what) {
    char *stop = nullptr;
    errno = 0;
    const long long value = std::strtoll(text, &stop, 10);
    const bool whole = stop != text && *stop == '\0' && errno != ERANGE;
    if (!whole || value <= 0) usage_error(what + " must be positive");
    return value;
}

int positive_int(const char *text, const std::string &what) {
    const long long value = positive_count(text, what);
    if (value > std::numeric_limits<int>::max()) usage_error(what + " exceeds GPU limit");
    return static_cast<int>(value);
}

Rational real_bound(const char *text, const std::string &what) {
    Rational value;
    std::string problem;
    if (!parse_real(text, what, value, problem)) usage_error(problem);
    return value;
}

// Whitespace-separated tokens of the coefficient argument, one leading '+' of
// each token dropped.
std::vector<std::string> coefficient_tokens(const char *text) {
    std::vector<std::string> tokens;
    const std::string s(text);
    std::size_t i = 0;
    while (i < s.size()) {
        while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i;
        const std::size_t begin = i;
        while (i < s.size() && !std::isspace(static_cast<unsigned char>(s[i]))) ++i;
        if (i > begin) tokens.push_back(s.substr(begin, i - begin));
    }
    for (auto &t : tokens)
        if (t[0] == '+') t.erase(t.begin());
    return tokens;
}

// Sign and digits of a decimal integer token: whether it is one, and whether
// its digits are all zero.
struct IntegerShape {
    bool integer;
    bool zero;
};

IntegerShape shape_of(const std::string &token) {
    const bool signed_token = !token.empty() && (token[0] == '+' || token[0] == '-');
    const auto digits = token.begin() + (signed_token ? 1 : 0);
    const bool any = digits != token.end();
    const bool all_digits = std::all_of(digits, token.end(), [](char c) { return c >= '0' && c <= '9'; });
    const bool all_zero = std::all_of(digits, token.end(), [](char c) { return c == '0'; });
    return {any && all_digits, all_zero};
}

void check_coefficients(const std::vector<std::string> &tokens) {
    if (tokens.size() < 2 || tokens.size() > kMostCoefficients)
        usage_error("supported polynomial degrees are 1 through 100");
    if (!std::all_of(tokens.begin(), tokens.end(),
                     [](const std::string &t) { return shape_of(t).integer; }))
        usage_error("coefficients must be decimal integers");
    if (shape_of(tokens.back()).zero) usage_error("leading coefficient must be nonzero");
}

// ---------------------------------------------------------------------------
// Option table and dispatcher

enum class Action {
    LowerDenominator, UpperDenominator, OpenInterval, CloseInterval, HideInfinity, ShowInfinity,
    HideOrdinates, ShowOrdinates, HidePoints, ShowPoints, Format, Prefix, Separator, Suffix,
    Devices, BatchSize, SquareDenominators, SievePlan, HostVerifyOnly, Quiet, Verbose,
    FirstPointOnly, NoEffect
};

struct OptionEntry {
    const char *flag;
    Action action;
};

constexpr OptionEntry kOptionTable[] = {
    {"-dl", Action::LowerDenominator}, {"-du", Action::UpperDenominator},
    {"-l", Action::OpenInterval},      {"-u", Action::CloseInterval},
    {"-i", Action::HideInfinity},      {"-I", Action::ShowInfinity},
    {"-y", Action::HideOrdinates},     {"-Y", Action::ShowOrdinates},
    {"-z", Action::HidePoints},        {"-Z", Action::ShowPoints},
    {"-f", Action::Format},            {"-fs", Action::Prefix},
    {"-fm", Action::Separator},        {"-fe", Action::Suffix},
    {"--devices", Action::Devices},    {"--batch-size", Action::BatchSize},
    {"--square-denominators", Action::SquareDenominators},
    {"--sieve-plan", Action::SievePlan},
    {"--host-verify-only", Action::HostVerifyOnly},
    {"-q", Action::Quiet},             {"-v", Action::Verbose},
    {"-1", Action::FirstPointOnly},
    // CPU-side switches of ratpoints; they do not change the searched set.
    {"-s", Action::NoEffect}, {"-k", Action::NoEffect}, {"-K", Action::NoEffect},
    {"-j", Action::NoEffect}, {"-J", Action::NoEffect},
};

class ArgumentReader {
public:
    ArgumentReader(int argc, char **argv, int start) : argc_(argc), argv_(argv), at_(start) {}
    bool done() const { return at_ >= argc_; }
    std::string take_flag() { return argv_[at_++]; }
    const char *take_value(const std::string &flag) {
        if (done()) usage_error(flag + " requires an argument");
        return argv_[at_++];
    }

private:
    int argc_;
    char **argv_;
    int at_;
};

// Interval state across -l / -u: an -l waits for its -u; an -l left open at
// the end becomes [lower, +infinity).
struct IntervalBuilder {
    bool open = false;
    Rational lower;

    void begin(const Rational &bound) {
        open = true;
        lower = bound;
    }
    void close(const Rational &upper, std::vector<SearchInterval> &out) {
        if (open && Rational::compare(lower, upper) > 0)
            usage_error("interval lower bound exceeds upper bound");
        if (!out.empty()) {
            const SearchInterval &prev = out.back();
            const bool ordered = open && !prev.upper_infinite && Rational::compare(lower, prev.upper) >= 0;
            if (!ordered) usage_error("search intervals must be ordered");
        }
        SearchInterval iv;
        iv.lower_infinite = !open;
        if (open) iv.lower = lower;
        iv.upper = upper;
        out.push_back(iv);
        open = false;
    }
    void finish(std::vector<SearchInterval> &out) {
        if (!open) return;
        SearchInterval iv;
        iv.lower = lower;
        iv.upper_infinite = true;
        out.push_back(iv);
        open = false;
    }
};

void apply(Action action, const std::string &flag, ArgumentReader &args, IntervalBuilder &intervals,
           Invocation &inv) {
    SearchOptions &s = inv.search;
    RenderSettings &r = inv.render;
    switch (action) {
    case Action::LowerDenominator: s.first = positive_int(args.take_value(flag), "lower denominator"); break;
    case Action::UpperDenominator: s.last = positive_int(args.take_value(flag), "upper denominator"); break;
    case Action::OpenInterval:
        // an unmatched -l is reported before this one's argument is read
        if (intervals.open) usage_error("interval lower bound without upper bound");
        intervals.begin(real_bound(args.take_value(flag), "interval lower bound"));
        break;
    case Action::CloseInterval:
        intervals.close(real_bound(args.take_value(flag), "interval upper bound"), s.intervals);
        break;
    case Action::HideInfinity: s.include_infinity = false; break;
    case Action::ShowInfinity: s.include_infinity = true; break;
    case Action::HideOrdinates: r.ordinates = false; break;
    case Action::ShowOrdinates: r.ordinates = true; break;
    case Action::HidePoints: r.points = false; break;
    case Action::ShowPoints: r.points = true; break;
    case Action::Format: r.format = args.take_value(flag); break;
    case Action::Prefix: r.before = args.take_value(flag); break;
    case Action::Separator: r.between = args.take_value(flag); break;
    case Action::Suffix: r.after = args.take_value(flag); break;
    case Action::Devices: s.devices = parse_device_selection(args.take_value(flag)); break;
    case Action::BatchSize:
        s.batch_size = positive_int(args.take_value(flag), "denominator batch size");
        if (s.batch_size > kLargestBatch) usage_error("--batch-size must not exceed 65536");
        break;
    case Action::SquareDenominators: s.square = true; break;
    case Action::SievePlan: {
        const std::string plan = args.take_value(flag);
        if (plan == "fast") s.plan = PlanKind::fast;
        else if (plan == "reference") s.plan = PlanKind::reference;
        else usage_error("--sieve-plan must be reference or fast");
        break;
    }
    case Action::HostVerifyOnly: s.device_preverify = false; break;
    case Action::Quiet: inv.quiet = true; break;
    case Action::Verbose: inv.verbose = true; break;
    case Action::FirstPointOnly: inv.first_point_only = true; break;
    case Action::NoEffect: break;
    }
}

Invocation read_invocation(int argc, char **argv) {
    if (argc < 3) usage_error("Usage: ratpoints_gpu 'c0 c1 ... cn' HEIGHT [OPTIONS]");
    Invocation inv;
    SearchOptions &s = inv.search;
    s.coefficients = coefficient_tokens(argv[1]);
    s.numerator_bound = positive_count(argv[2], "maximum height");
    if (s.numerator_bound > kHeightCeiling) usage_error("maximum height exceeds safe GPU limit");
    s.last = std::min<long long>(s.numerator_bound, std::numeric_limits<int>::max());

    ArgumentReader args(argc, argv, 3);
    IntervalBuilder intervals;
    while (!args.done()) {
        const std::string flag = args.take_flag();
        const auto *entry = std::find_if(std::begin(kOptionTable), std::end(kOptionTable),
                                         [&](const OptionEntry &e) { return flag == e.flag; });
        if (entry == std::end(kOptionTable)) usage_error("unsupported ratpoints option: " + flag);
        apply(entry->action, flag, args, intervals, inv);
    }
    intervals.finish(s.intervals);

    s.last = std::min(s.last, s.numerator_bound);
    if (s.square) s.last = std::min<long long>(s.last, kSquareDenominatorCeiling);
    if (s.first > s.last) usage_error("empty denominator range");
    check_coefficients(s.coefficients);
    return inv;
}

// ---------------------------------------------------------------------------
// Help, device listing and metrics

constexpr char kHelpText[] =
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

void show_help(std::FILE *to) {
    if (std::fputs(kHelpText, to) == EOF) throw std::runtime_error("failed to write help output");
}

void describe_device(std::FILE *to, const GpuDevice &g) {
    std::fprintf(to, "device=%d name=\"%s\" compute=%d.%d sm=%d memory_mib=%llu pci=%s\n", g.id,
                 g.name.c_str(), g.major, g.minor, g.multiprocessors, g.memory_bytes >> 20,
                 g.pci_bus_id.c_str());
}

// The -v line: key=value fields in the reference's order and formats (the
// reference's benchmark harness parses them), then one pair of lines per GPU.
void report_metrics(const SearchMetrics &m) {
    struct Field {
        const char *key;
        bool real;
        double x;
        unsigned long long n;
    };
    const Field fields[] = {
        {"wall_ms", true, m.wall_ms, 0},
        {"devices", false, 0, m.devices.size()},
        {"denominators", false, 0, m.denominator_count},
        {"basis_ms", true, m.basis_ms, 0},
        {"sieve_ms", true, m.sieve_ms, 0},
        {"words", false, 0, m.word_count},
        {"initial_mask_gbs", true, m.initial_mask_gbs(), 0},
        {"survivors", false, 0, m.modular_survivors},
        {"exact_survivors", false, 0, m.exact_survivors},
        {"plan_ms", true, m.plan_ms, 0},
        {"workspace_ms", true, m.workspace_ms, 0},
        {"basis_wall_ms", true, m.basis_wall_ms, 0},
        {"survivor_setup_ms", true, m.survivor_setup_ms, 0},
        {"verification_ms", true, m.verification_ms, 0},
        {"sieve_wall_ms", true, m.sieve_wall_ms, 0},
    };
    std::string line;
    char buf[64];
    for (const Field &f : fields) {
        if (f.real) std::snprintf(buf, sizeof buf, "%s=%.3f", f.key, f.x);
        else std::snprintf(buf, sizeof buf, "%s=%llu", f.key, f.n);
        if (!line.empty()) line.push_back(' ');
        line += buf;
    }
    std::fprintf(stderr, "%s\n", line.c_str());
    for (const DeviceMetrics &d : m.devices) {
        describe_device(stderr, d.device);
        std::fprintf(stderr, "gpu=%d denominators=%llu batches=%llu basis_ms=%.3f sieve_ms=%.3f\n",
                     d.device.id, d.denominator_count, d.batches, d.basis_ms, d.sieve_ms);
    }
}

// ---------------------------------------------------------------------------
// Program flow

enum class Request { HelpOnStderr, Help, ListDevices, Search };

Request classify(int argc, char **argv) {
    if (argc <= 1) return Request::HelpOnStderr;
    if (argc == 2 && std::strcmp(argv[1], "--help") == 0) return Request::Help;
    if (argc == 2 && std::strcmp(argv[1], "--list-devices") == 0) return Request::ListDevices;
    return Request::Search;
}

int search_and_print(int argc, char **argv) {
    const Invocation inv = read_invocation(argc, argv);
    PointSearch search(inv.search);  // validates before anything is written
    PointPrinter printer(inv.render, stdout);
    const bool keep_going = !inv.first_point_only;
    const SearchMetrics metrics = search.run([&](const PointPair &p) {
        printer.point(p.numerator, p.ordinate, p.denominator, keep_going);
        return keep_going;
    });
    printer.close();
    const bool benchmark_env = std::getenv("RATPOINTS_GPU_BENCHMARK") != nullptr;
    if (benchmark_env || (inv.verbose && !inv.quiet)) report_metrics(metrics);
    return 0;
}

}  // namespace

int run_cli(int argc, char **argv) {
    try {
        switch (classify(argc, argv)) {
        case Request::HelpOnStderr:
            show_help(stderr);
            return 1;
        case Request::Help:
            show_help(stdout);
            return 0;
        case Request::ListDevices:
            for (const GpuDevice &g : available_gpu_devices()) describe_device(stdout, g);
            return std::fflush(stdout) == EOF ? 1 : 0;
        case Request::Search:
            return search_and_print(argc, argv);
        }
        return 1;
    } catch (const std::exception &error) {
        std::fflush(stdout);
        std::fprintf(stderr, "%s\n", error.what());
        return 1;
    }
}

}  // namespace rpg
