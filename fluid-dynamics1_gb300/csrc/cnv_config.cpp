// cnv_config.cpp -- cnavier's configuration format (src/config.c, include/config.h).
//
// Same defaults (src/config.c:47-87), same line format and parsing rules
// (src/config.c:106-214): lines starting with '\n', '#' or ';' are skipped, a line is split by
// sscanf("%63[^=]=%63s"), key and value are trimmed of spaces/tabs/CR/LF, integer keys use
// atoi and real keys atof (so "Lx = 1.5" reads as 1), and an unknown key prints the same
// warning and is ignored. Extension keys (see cnv_config in cnv.h) default to the reference's
// behaviour; an unmodified reference parser warns about them and ignores them.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <strings.h>

#include "cnv_internal.h"

namespace {

int parse_precision(const char* v) {
    if (!strcasecmp(v, "fp64") || !strcmp(v, "0")) return CNV_PREC_FP64;
    if (!strcasecmp(v, "fp64_fma") || !strcmp(v, "1")) return CNV_PREC_FP64_FMA;
    if (!strcasecmp(v, "mixed") || !strcmp(v, "2")) return CNV_PREC_MIXED;
    return -1;
}

int parse_init(const char* v) {
    if (!strcasecmp(v, "reference") || !strcasecmp(v, "zero") || !strcmp(v, "0")) return CNV_INIT_REFERENCE;
    if (!strcasecmp(v, "noise") || !strcmp(v, "1")) return CNV_INIT_NOISE;
    return -1;
}

}  // namespace

extern "C" int cnv_config_default(cnv_config* c) {
    if (!c) return CNV_BAD_ARG;
    std::memset(c, 0, sizeof(*c));
    c->Re = 1000.0;
    c->Lx = 1;
    c->Ly = 1;
    c->nx = 64;
    c->ny = 64;
    c->dt = 0.005;
    c->tf = 20.0;
    c->max_co = 1.0;
    c->order = 6;
    c->poisson_max_it = 10000;
    c->poisson_tol = 1E-3;
    c->output_interval = 10;
    c->poisson_type = 2;
    c->openmp_enabled = 1;  // the OPENMP_ENABLED build's default: red-black sweeps
    c->ui = 0.0;
    c->vi = 0.0;
    c->u1 = 0.0;
    c->u2 = 0.0;
    c->u3 = 0.0;
    c->u4 = 1.0;
    c->v1 = 0.0;
    c->v2 = 0.0;
    c->v3 = 0.0;
    c->v4 = 0.0;
    c->sor_omega = 0.0;
    c->nsteps = 0;
    c->precision = CNV_PREC_FP64;
    c->mixed_rtol = 0.0;
    c->init_field = CNV_INIT_REFERENCE;
    c->seed = 0;
    c->init_sigma = 0.1;
    c->init_smooth_passes = 8;
    c->device = 0;
    return CNV_OK;
}

extern "C" int cnv_config_set(cnv_config* c, const char* key, const char* v) {
    if (!c || !key || !v) return CNV_BAD_ARG;
    // include/config.h field by field (src/config.c:151-207)
    if (!strcmp(key, "Re")) c->Re = atof(v);
    else if (!strcmp(key, "Lx")) c->Lx = atoi(v);
    else if (!strcmp(key, "Ly")) c->Ly = atoi(v);
    else if (!strcmp(key, "nx")) c->nx = atoi(v);
    else if (!strcmp(key, "ny")) c->ny = atoi(v);
    else if (!strcmp(key, "dt")) c->dt = atof(v);
    else if (!strcmp(key, "tf")) c->tf = atof(v);
    else if (!strcmp(key, "max_co")) c->max_co = atof(v);
    else if (!strcmp(key, "order")) c->order = atoi(v);
    else if (!strcmp(key, "poisson_max_it")) c->poisson_max_it = atoi(v);
    else if (!strcmp(key, "poisson_tol")) c->poisson_tol = atof(v);
    else if (!strcmp(key, "output_interval")) c->output_interval = atoi(v);
    else if (!strcmp(key, "poisson_type")) c->poisson_type = atoi(v);
    else if (!strcmp(key, "openmp_enabled")) c->openmp_enabled = atoi(v);
    else if (!strcmp(key, "ui")) c->ui = atof(v);
    else if (!strcmp(key, "vi")) c->vi = atof(v);
    else if (!strcmp(key, "u1")) c->u1 = atof(v);
    else if (!strcmp(key, "u2")) c->u2 = atof(v);
    else if (!strcmp(key, "u3")) c->u3 = atof(v);
    else if (!strcmp(key, "u4")) c->u4 = atof(v);
    else if (!strcmp(key, "v1")) c->v1 = atof(v);
    else if (!strcmp(key, "v2")) c->v2 = atof(v);
    else if (!strcmp(key, "v3")) c->v3 = atof(v);
    else if (!strcmp(key, "v4")) c->v4 = atof(v);
    // extensions
    else if (!strcmp(key, "sor_omega")) c->sor_omega = atof(v);
    else if (!strcmp(key, "nsteps")) c->nsteps = atoi(v);
    else if (!strcmp(key, "precision")) {
        int p = parse_precision(v);
        if (p < 0) return CNV_BAD_ARG;
        c->precision = p;
    } else if (!strcmp(key, "mixed_rtol")) c->mixed_rtol = atof(v);
    else if (!strcmp(key, "init_field")) {
        int p = parse_init(v);
        if (p < 0) return CNV_BAD_ARG;
        c->init_field = p;
    } else if (!strcmp(key, "seed")) c->seed = strtoull(v, nullptr, 0);
    else if (!strcmp(key, "init_sigma")) c->init_sigma = atof(v);
    else if (!strcmp(key, "init_smooth_passes")) c->init_smooth_passes = atoi(v);
    else if (!strcmp(key, "device")) c->device = atoi(v);
    else if (!strcmp(key, "solver_blocks")) c->solver_blocks = atoi(v);
    else if (!strcmp(key, "mixed_inner_sweeps")) c->mixed_inner_sweeps = atoi(v);
    else if (!strcmp(key, "mixed_max_outer")) c->mixed_max_outer = atoi(v);
    else if (!strcmp(key, "sor_blocking")) c->sor_blocking = atoi(v);
    else if (!strcmp(key, "mixed_warm_start")) c->mixed_warm_start = atoi(v);
    else if (!strcmp(key, "solver_timeout_ms")) c->solver_timeout_ms = atoi(v);
    else return CNV_BAD_ARG;
    return CNV_OK;
}

extern "C" int cnv_config_load(const char* path, cnv_config* c) {
    if (!c) return CNV_BAD_ARG;
    cnv_config_default(c);  // start from the defaults, src/config.c:107
    if (!path) return CNV_BAD_ARG;
    FILE* f = std::fopen(path, "r");
    if (!f) {
        std::printf("Error: Could not open configuration file '%s'\n", path);
        std::printf("Using default configuration.\n");
        std::fflush(stdout);
        return CNV_IO_ERROR;
    }
    char line[256], key[64], value[64];
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '\n' || line[0] == '#' || line[0] == ';') continue;
        if (std::sscanf(line, "%63[^=]=%63s", key, value) != 2) continue;
        char* k = key;
        while (*k == ' ' || *k == '\t') ++k;
        char* ke = k + std::strlen(k) - 1;
        while (ke > k && (*ke == ' ' || *ke == '\t' || *ke == '\n' || *ke == '\r')) *ke-- = '\0';
        char* v = value;
        while (*v == ' ' || *v == '\t') ++v;
        char* ve = v + std::strlen(v) - 1;
        while (ve > v && (*ve == ' ' || *ve == '\t' || *ve == '\n' || *ve == '\r')) *ve-- = '\0';
        if (cnv_config_set(c, k, v) == CNV_BAD_ARG) {
            // unknown key (or an extension value that does not parse): warn and go on
            std::printf("Warning: Unknown configuration parameter '%s'\n", k);
        }
    }
    std::fclose(f);
    std::fflush(stdout);
    return CNV_OK;
}

extern "C" int cnv_config_steps(const cnv_config* c) {
    if (!c) return -1;
    if (c->nsteps > 0) return c->nsteps;
    int it_max = (int)((c->tf / c->dt) - 1);  // src/main.c:162
    return it_max + 1 > 0 ? it_max + 1 : 0;
}
