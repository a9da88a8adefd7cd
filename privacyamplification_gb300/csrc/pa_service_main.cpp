// pa_service_main.cpp -- the `pa_service` executable: the reference's program entry
// (PrivacyAmplification.cu:1394-1680) on the GB300 engine.
//
//   pa_service [config.yaml] [--blocks K]
//
// Reads the config (default ./config.yaml; exit 102 when unreadable), then serves blocks until killed
// or until K results have been sent.  The exit code is pa_service_run's.
#include "../../include/pa_service.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>

int main(int argc, char** argv) {
    const char* path = "config.yaml";
    long long blocks = -1;
    for (int i = 1; i < argc; ++i) {
        if (std::strcmp(argv[i], "--blocks") == 0 && i + 1 < argc) blocks = std::atoll(argv[++i]);
        else path = argv[i];
    }
    pa_service_config cfg;
    pa_service_config_default(&cfg);
    std::printf("# Reading %s...\n", path);
    if (pa_service_config_load(path, &cfg) != 0) {
        std::printf("Can't open file %s => terminating!\n", path);
        return 102;
    }
    std::printf("# PrivacyAmplification (GB300 engine) with %u bits\n", 1u << cfg.factor_exp);
    std::fflush(stdout);
    return pa_service_run(&cfg, blocks);
}
