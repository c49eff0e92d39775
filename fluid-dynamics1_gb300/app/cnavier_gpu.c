/*
 * cnavier_gpu.c -- the reference program's command line and outputs, with the time loop on
 * the GPU through libcnv.
 *
 * Usage as src/main.c:36-90: no argument (default configuration), a configuration file, or a
 * configuration file and a run name (outputs under ./output/<run name>). Writes the same log
 * (./output/logs/<run name>.txt: header of src/main.c:255-271, per step the Poisson line and
 * the two progress lines of src/main.c:401-414, timing summary of :455-459) and the same VTK
 * files every output_interval steps (stream-function, vorticity, x-velocity, y-velocity with
 * one shared counter, src/main.c:429-436, src/utils.c:38-99). Field values, iteration counts,
 * stop norms and continuity values equal the reference's OpenMP (red-black) build bit for bit;
 * timings are this program's.
 *
 * Steps between two outputs run as one enqueued call; while the GPU runs them, the host formats
 * the previous output's files (the fields are copied out before the call is enqueued).
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>

#include "cnv.h"

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void usage(const char *prog) {
    printf("Usage: %s [config_file] [run_name]\n", prog);
    printf("  no arguments         run with the default configuration\n");
    printf("  config_file          key = value configuration (same format as the reference)\n");
    printf("  config_file run_name outputs under ./output/<run_name>, log ./output/logs/<run_name>.txt\n");
}

static int mkdirs(const char *path) {
    char tmp[512];
    size_t i, len = strlen(path);
    if (len >= sizeof tmp) return -1;
    memcpy(tmp, path, len + 1);
    for (i = 1; i <= len; ++i)
        if (tmp[i] == '/' || tmp[i] == '\0') {
            char c = tmp[i];
            tmp[i] = '\0';
            mkdir(tmp, 0777);
            tmp[i] = c;
        }
    return 0;
}

typedef struct {
    double *w, *u, *v, *psi;
} fields;

static void write_vtk(const char *dir, int *count, const fields *f, int n) {
    /* src/main.c:431-434 order */
    const char *titles[4] = {"stream-function", "vorticity", "x-velocity", "y-velocity"};
    const double *data[4] = {f->psi, f->w, f->u, f->v};
    int k;
    for (k = 0; k < 4; ++k) {
        char name[600];
        snprintf(name, sizeof name, "%s/%s-1-%d.vtk", dir, titles[k], *count);
        if (cnv_write_vtk(dir, titles[k], *count, data[k], n, n) != CNV_OK) {
            printf("\nError while opening file: %s\n", name);
            exit(1);
        }
        printf("%s\n", name);
        ++*count;
    }
}

int main(int argc, char **argv) {
    cnv_config cfg;
    char output_dir[256] = "./output";
    char run_name[256] = "default";
    char log_filename[1024];
    FILE *log_file;
    cnv_state *s = NULL;
    int rc, it_max, nsteps, t, n, vtk_count = 0, interval;
    const double start = now_s();
    double sim_start;
    fields cur;
    int pending = 0;
    cnv_step_info *info;
    char *line;
    const size_t line_len = 4096;

    cnv_config_default(&cfg);
    if (argc == 1) {
        printf("No configuration file specified. Using default values.\n");
    } else if (argc == 2) {
        if (!strcmp(argv[1], "--help") || !strcmp(argv[1], "-h")) {
            usage(argv[0]);
            return 0;
        }
        cnv_config_load(argv[1], &cfg);
    } else if (argc == 3) {
        cnv_config_load(argv[1], &cfg);
        snprintf(output_dir, sizeof output_dir, "./output/%s", argv[2]);
        printf("Using output directory: %s\n", output_dir);
        snprintf(run_name, sizeof run_name, "%s", argv[2]);
    } else {
        printf("Error: Too many arguments.\n");
        usage(argv[0]);
        return 1;
    }
    it_max = (int)((cfg.tf / cfg.dt) - 1); /* src/main.c:162 */
    nsteps = cnv_config_steps(&cfg);
    interval = cfg.output_interval > 0 ? cfg.output_interval : 1;
    rc = cnv_create(&cfg, &s);
    if (rc != CNV_OK) {
        printf("%s\n", cnv_last_error());
        return 1;
    }
    n = cnv_grid_size(s);
    printf("%s: %dx%d, Re %.2f, %d steps on the GPU (%s)\n", argv[0], n, n, cfg.Re, nsteps, cnv_version());

    mkdirs("./output/logs");
    snprintf(log_filename, sizeof log_filename, "./output/logs/%s.txt", run_name);
    log_file = fopen(log_filename, "w");
    if (!log_file) {
        printf("Warning: Could not create log file %s. Logging to console instead.\n", log_filename);
        log_file = stdout;
    } else {
        printf("Logging simulation progress to: %s\n", log_filename);
    }
    fprintf(log_file, "=== Fluid Dynamics Simulation Log ===\n");
    fprintf(log_file, "Run name: %s\n", run_name);
    fprintf(log_file, "Output directory: %s\n", output_dir);
    fprintf(log_file, "Reynolds number: %.2f\n", cfg.Re);
    fprintf(log_file, "Grid size: %dx%d\n", cfg.nx, cfg.ny);
    fprintf(log_file, "Time step: %.6f\n", cfg.dt);
    fprintf(log_file, "Final time: %.2f\n", cfg.tf);
    fprintf(log_file, "Max iterations: %d\n", it_max + 1);
    fprintf(log_file, "OpenMP enabled: %s\n", cfg.openmp_enabled ? "Yes" : "No");
    fprintf(log_file, "=====================================\n\n");
    fflush(log_file);

    cur.w = (double *)malloc(sizeof(double) * (size_t)n * n * 4);
    info = (cnv_step_info *)malloc(sizeof(cnv_step_info) * (size_t)interval);
    line = (char *)malloc(line_len);
    if (!cur.w || !info || !line) {
        printf("** Error: insufficient memory **\n");
        return 1;
    }
    cur.u = cur.w + (size_t)n * n;
    cur.v = cur.u + (size_t)n * n;
    cur.psi = cur.v + (size_t)n * n;

    sim_start = now_s();
    for (t = 0; t < nsteps;) {
        /* the reference writes VTK after step t when t % output_interval == 0 */
        const int k = (t % interval == 0) ? 1 : interval - t % interval;
        const int chunk = k < nsteps - t ? k : nsteps - t;
        double t0 = now_s(), dt_call;
        int i, status;
        rc = cnv_step_async(s, chunk);
        if (pending) { /* format the last output while the GPU runs this chunk */
            write_vtk(output_dir, &vtk_count, &cur, n);
            pending = 0;
        }
        if (rc == CNV_OK) rc = cnv_sync(s, info, chunk);
        dt_call = now_s() - t0;
        for (i = 0; i < chunk; ++i) {
            status = info[i].status;
            if (cnv_format_step_log(&info[i], t + i, cfg.dt, it_max, dt_call / chunk, now_s() - sim_start, line,
                                    line_len) == CNV_OK) {
                fputs(line, log_file);
                fflush(log_file);
            }
            if (status != CNV_OK) {
                if (status != CNV_NOT_CONVERGED) printf("%s\n", cnv_last_error());
                return 1; /* src/poisson.c:284: exit(1) */
            }
        }
        if (rc != CNV_OK) {
            printf("%s\n", cnv_last_error());
            return 1;
        }
        t += chunk;
        if ((t - 1) % interval == 0) {
            cnv_get_fields(s, cur.w, cur.u, cur.v, cur.psi);
            pending = 1;
        }
    }
    if (pending) write_vtk(output_dir, &vtk_count, &cur, n);
    printf("Simulation complete!\n");
    {
        const double end = now_s();
        fprintf(log_file, "\n=== Timing Summary ===\n");
        fprintf(log_file, "Setup time: %.4f seconds\n", sim_start - start);
        fprintf(log_file, "Simulation time: %.2f seconds\n", end - sim_start);
        fprintf(log_file, "Total program time: %.2f seconds\n", end - start);
    }
    if (log_file != stdout) fclose(log_file);
    cnv_destroy(s);
    free(cur.w);
    free(info);
    free(line);
    return 0;
}
