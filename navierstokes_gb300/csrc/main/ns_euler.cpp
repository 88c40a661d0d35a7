// ns_euler -- the euler.f90 program (euler.f90:36-206) with the time step on
// the GPU: reads dados.in, runs iter = 0..maxit, writes temp1_D60.dat ..
// temp3_D60.dat every ctd steps and contorno_<n>.dat every cgd steps.
//
//   ns_euler [dados.in] [--outdir DIR] [--nk 4|5] [--device N] [--maxit N]
//            [--no-contorno] [--quiet]
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "ns_gb300.h"

static int usage()
{
    std::fprintf(stderr,
                 "usage: ns_euler [dados.in] [--outdir DIR] [--nk 4|5] [--device N] "
                 "[--maxit N] [--no-contorno] [--quiet]\n");
    return 2;
}

int main(int argc, char **argv)
{
    const char *dados = "dados.in", *outdir = ".";
    int nk = 5, device = 0, maxit = -1, flags = 0;
    for (int a = 1; a < argc; a++) {
        const char *s = argv[a];
        auto value = [&](void) -> const char * { return (a + 1 < argc) ? argv[++a] : nullptr; };
        if (!std::strcmp(s, "--outdir")) {
            if (!(outdir = value())) return usage();
        } else if (!std::strcmp(s, "--nk")) {
            const char *v = value();
            if (!v) return usage();
            nk = std::atoi(v);
        } else if (!std::strcmp(s, "--device")) {
            const char *v = value();
            if (!v) return usage();
            device = std::atoi(v);
        } else if (!std::strcmp(s, "--maxit")) {
            const char *v = value();
            if (!v) return usage();
            maxit = std::atoi(v);
        } else if (!std::strcmp(s, "--no-contorno")) {
            flags |= NS_RUN_NO_CONTORNO;
        } else if (!std::strcmp(s, "--quiet")) {
            flags |= NS_RUN_QUIET;
        } else if (s[0] == '-') {
            return usage();
        } else {
            dados = s;
        }
    }
    const int rc = ns_run_euler(dados, outdir, nk, device, maxit, flags);
    if (rc != NS_OK) {
        std::fprintf(stderr, "ns_euler: %s\n", ns_last_error(nullptr));
        return 1;
    }
    return 0;
}
