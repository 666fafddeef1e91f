// Drives rpg::PointPrinter (csrc/point_format.cpp) without a search: the
// output settings come from argv, the points from stdin ("x y z" per line),
// and the printed bytes go to stdout, for comparison with the oracle's
// restatement of the reference's formatter.
//   point_format_check POINTS(0|1) ORDINATES(0|1) CONJUGATES(0|1) FORMAT BEFORE BETWEEN AFTER
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <string>

#include "point_format.hpp"

int main(int argc, char **argv) {
    if (argc != 8) return 2;
    rpg::RenderSettings r;
    r.points = argv[1][0] == '1';
    r.ordinates = argv[2][0] == '1';
    const bool conjugates = argv[3][0] == '1';
    r.format = argv[4];
    r.before = argv[5];
    r.between = argv[6];
    r.after = argv[7];
    rpg::PointPrinter printer(r, stdout);
    long long x = 0, z = 0;
    std::string y;
    while (std::cin >> x >> y >> z) printer.point(x, y, z, conjugates);
    printer.close();
    return 0;
}
