// visgpu.cpp -- command-line driver with the reference's behaviour
// (Main.cpp:4-11): reads config.txt from the working directory (or the path
// given as the first argument) and reconstructs every configured frame.
#include <cstdio>
#include <cstring>

#include "pms.h"

int main(int argc, char** argv) {
    const char* cfg = "config.txt";
    int verbose = 1;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "-q")) verbose = 0;
        else if (!strcmp(argv[i], "-h") || !strcmp(argv[i], "--help")) {
            printf("usage: %s [-q] [config.txt]\n", argv[0]);
            return 0;
        } else cfg = argv[i];
    }
    pms_status st = pms_run_config(cfg, verbose);
    if (st != PMS_OK) fprintf(stderr, "visgpu: %s\n", pms_status_string(st));
    return st == PMS_OK ? 0 : 1;
}
