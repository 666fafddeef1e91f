#include "point_format.hpp"

#include <algorithm>
#include <stdexcept>

namespace rpg {

namespace {

// Backslash escapes of -f/-fs/-fm/-fe: \n and \t become the control
// characters, \% a percent sign that is never a field marker, any other
// backslash pair and a trailing backslash stay as written.
struct TextUnit {
    char ch;
    bool escaped_percent;
};

std::vector<TextUnit> unescape(const std::string &raw) {
    std::vector<TextUnit> units;
    for (std::size_t i = 0; i < raw.size(); ++i) {
        if (raw[i] == '\\' && i + 1 < raw.size()) {
            const char next = raw[++i];
            if (next == 'n') units.push_back({'\n', false});
            else if (next == 't') units.push_back({'\t', false});
            else if (next == '%') units.push_back({'%', true});
            else {
                units.push_back({'\\', false});
                units.push_back({next, false});
            }
        } else {
            units.push_back({raw[i], false});
        }
    }
    return units;
}

// -fs, -fm and -fe are written unescaped, except that an escaped percent sign
// stays the byte 0x01 there: the reference substitutes it back to '%' only
// inside point lines (src/output_formatter.cpp:55-59), and its output bytes
// are the contract.
std::string literal_text(const std::string &raw) {
    std::string out;
    for (const TextUnit &u : unescape(raw)) out.push_back(u.escaped_percent ? '\x01' : u.ch);
    return out;
}

}  // namespace

PointTemplate::PointTemplate(const std::string &raw, bool ordinates) {
    const std::vector<TextUnit> units = unescape(raw);
    for (std::size_t i = 0; i < units.size(); ++i) {
        const TextUnit &u = units[i];
        if (u.ch != '%' || u.escaped_percent || i + 1 == units.size()) {
            literal(u.ch);
            continue;
        }
        const TextUnit &m = units[++i];
        // %y is a field only while ordinates are shown: under -y it stays
        // the two characters "%y", as in the reference
        const Field f = m.escaped_percent          ? Field::Text
                        : m.ch == 'x'              ? Field::Numerator
                        : m.ch == 'y' && ordinates ? Field::Ordinate
                        : m.ch == 'z'              ? Field::Denominator
                                                   : Field::Text;
        if (f == Field::Text) {
            literal('%');
            literal(m.ch);
        } else {
            pieces_.push_back({f, {}});
        }
    }
}

void PointTemplate::literal(char c) {
    if (pieces_.empty() || pieces_.back().field != Field::Text) pieces_.push_back({Field::Text, {}});
    pieces_.back().text.push_back(c);
}

std::string PointTemplate::render(long long x, const std::string &y, long long z) const {
    std::string line;
    for (const Piece &p : pieces_) {
        switch (p.field) {
        case Field::Text: line += p.text; break;
        case Field::Numerator: line += std::to_string(x); break;
        case Field::Ordinate: line += y; break;
        case Field::Denominator: line += std::to_string(z); break;
        }
    }
    return line;
}

PointPrinter::PointPrinter(const RenderSettings &r, std::FILE *out)
    : out_(out), show_(r.points), ordinates_(r.ordinates),
      line_(r.format.empty() ? (r.ordinates ? "(%x : %y : %z)\\n" : "(%x : %z)\\n") : r.format,
            r.ordinates),
      between_(literal_text(r.between)), after_(literal_text(r.after)) {
    if (show_) put(literal_text(r.before));
}

void PointPrinter::point(long long x, const std::string &y, long long z, bool with_conjugate) {
    emit(x, y, z);
    if (with_conjugate && ordinates_ && y != "0") emit(x, "-" + y, z);
}

void PointPrinter::close() {
    if (closed_) return;
    put(after_);
    if (std::fflush(out_) == EOF) throw std::runtime_error("failed to flush standard output");
    closed_ = true;
}

void PointPrinter::emit(long long x, const std::string &y, long long z) {
    if (!show_) return;
    if (lines_++) put(between_);
    std::string text = line_.render(x, y, z);
    // a 0x01 byte written in the format itself prints as '%', as in the
    // reference, which marks escaped percent signs with that byte
    std::replace(text.begin(), text.end(), '\x01', '%');
    put(text);
}

void PointPrinter::put(const std::string &text) {
    if (std::fputs(text.c_str(), out_) == EOF) throw std::runtime_error("failed to write standard output");
}

}  // namespace rpg
