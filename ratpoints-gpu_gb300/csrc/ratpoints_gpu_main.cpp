// ratpoints_gpu executable: the ratpoints-compatible command line over librpgpu.
#include "cli.hpp"

int main(int argc, char **argv) { return rpg::run_cli(argc, argv); }
