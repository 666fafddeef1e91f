// Entry point of the ratpoints_gpu command line (src/main.cpp:48-85 in the
// reference): returns the process exit status.
#pragma once

namespace rpg {

int run_cli(int argc, char **argv);

}  // namespace rpg
