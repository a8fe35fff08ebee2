// boidsim_main.cpp -- entry point of the boidsim (all-pairs) and
// boidsim_grid (grid) executables, the reference targets built from
// src/main.cpp with src/boid_simulation.cpp or src/boid_simulation_grid.cpp.
// The engine is chosen at compile time, as the reference chooses it at link
// time: -DBOIDSIM_ENGINE=BOIDS_ENGINE_ALLPAIRS or BOIDS_ENGINE_GRID.
#include <iostream>
#include <string>

#include "boids.h"
#include "boids_cli.h"

#ifndef BOIDSIM_ENGINE
#error "define BOIDSIM_ENGINE"
#endif

int main(int argc, char **argv)
{
    boidscli::Args args;
    std::string err;
    switch (boidscli::parse_args(argc, argv, args, err)) {
    case boidscli::PARSE_HELP:
        std::cout << boidscli::usage(argv[0]) << std::endl;
        return 0;
    case boidscli::PARSE_ERROR:
        std::cout << err << std::endl;  // src/args.cpp:46-48 prints what() and exits
        return -1;
    default:
        break;
    }
    if (args.print_config) {
        std::cout << boidscli::format_config(args);
        return 0;
    }
    return boidscli::run(args, BOIDSIM_ENGINE, argv[0]);
}
