// Point output of the command line: the -f/-fs/-fm/-fe/-y/-z settings and the
// printer that writes a search's points with them.
//
// The bytes are the reference's (src/output_formatter.cpp:7-105): the -fs
// text when points are shown, one line per point and one for its conjugate
// (unless -y, or the ordinate is 0, or only the first point is asked for),
// the -fm text between lines, and the -fe text at the end even under -z.
// Default line format "(%x : %y : %z)\n", or "(%x : %z)\n" under -y.
#pragma once

#include <cstdio>
#include <string>
#include <vector>

namespace rpg {

struct RenderSettings {
    bool points = true;        // -z / -Z
    bool ordinates = true;     // -y / -Y
    std::string format;        // -f (empty: the default for the ordinate setting)
    std::string before, between, after;  // -fs, -fm, -fe
};

// A point line compiled once from the -f text: literal pieces and the %x,
// %y, %z fields.
class PointTemplate {
public:
    PointTemplate(const std::string &raw, bool ordinates);
    std::string render(long long x, const std::string &y, long long z) const;

private:
    enum class Field { Text, Numerator, Ordinate, Denominator };
    struct Piece {
        Field field;
        std::string text;
    };
    void literal(char c);

    std::vector<Piece> pieces_;
};

class PointPrinter {
public:
    PointPrinter(const RenderSettings &settings, std::FILE *out);
    // One verified point (x : y : z); its conjugate (x : -y : z) follows when
    // with_conjugate is set, ordinates are shown and y is not 0.
    void point(long long x, const std::string &y, long long z, bool with_conjugate);
    // The -fe text and a flush; later calls do nothing.
    void close();

private:
    void emit(long long x, const std::string &y, long long z);
    void put(const std::string &text);

    std::FILE *out_;
    bool show_, ordinates_;
    PointTemplate line_;
    std::string between_, after_;
    unsigned long long lines_ = 0;
    bool closed_ = false;
};

}  // namespace rpg
