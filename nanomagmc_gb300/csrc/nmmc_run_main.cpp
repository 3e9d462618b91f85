// `nmmc_run INPUT_FILE [outdir] [seed]`: the reference's `./run INPUT_FILE`
// (README: `mpirun -n N ./run INPUT`) on one GPU. Temps/, Fields/ and Js/ are read from the
// working directory, as the reference does.
#include <stdio.h>
#include <stdlib.h>

#include "../../include/nmmc.h"

int main(int argc, char** argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s INPUT_FILE [outdir] [seed]\n", argv[0]);
        return 2;
    }
    const char* out = argc > 2 ? argv[2] : "Output";
    unsigned long long seed = argc > 3 ? strtoull(argv[3], nullptr, 10) : 1ull;
    int rc = nmmc_run(argv[1], ".", out, seed, 1);
    if (rc) fprintf(stderr, "nmmc_run failed (%d): %s\n", rc, nmmc_last_error());
    return rc;
}
