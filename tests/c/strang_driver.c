/*
 * A time-stepping driver written only against the reference's C call surface
 * (C/spu_function.h:1-15): it replays the loop of C/mhd.c:59-124 (calcfl,
 * then x(F,A) T12 y(F,A) T13 z(F,A,A,F) T13 y(A,F) T12 x(A,F) with a
 * copy_matrix after every operator).  The same source links unchanged against
 * the reference's own C build (oracle/_ref) or against libmhd_gb300.so.
 *
 * usage: strang_driver in.bin out.bin nx ny nz nsteps cfl [device]
 *   in.bin : u (5*N floats) then b (3*N floats), N = nx*ny*nz
 *   out.bin: u, b after nsteps, then t (1 float)
 * With "device" (only when built with -DWITH_CUDA_MEMORY) the four arrays live
 * in cudaMalloc memory and the library works on them in place; otherwise they
 * are plain host arrays, as in the reference.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef WITH_CUDA_MEMORY
#include <cuda_runtime.h>
#endif

void fluidx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u, float *update_b,
            int iter);
void copy_matrix(float *u, float *b, int *nx, int *ny, int *nz, float *update_u, float *update_b);
void advectbyzx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u, float *update_b);
void transpose12(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz, int iter);
void transpose13(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz);
float calcfl(float *u, float *b, int *nx, int *ny, int *nz);

int main(int argc, char **argv)
{
    if (argc < 8) {
        fprintf(stderr, "usage: %s in.bin out.bin nx ny nz nsteps cfl [device]\n", argv[0]);
        return 2;
    }
    int nx = atoi(argv[3]), ny = atoi(argv[4]), nz = atoi(argv[5]), nsteps = atoi(argv[6]);
    double cfl = atof(argv[7]);
    int use_dev = argc > 8 && strcmp(argv[8], "device") == 0;
    size_t N = (size_t)nx * ny * nz;
    float *hu = malloc(N * 5 * sizeof(float)), *hb = malloc(N * 3 * sizeof(float));
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(hu, sizeof(float), N * 5, f) != N * 5 || fread(hb, sizeof(float), N * 3, f) != N * 3) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 1;
    }
    fclose(f);

    float *u = hu, *b = hb, *uu, *ub;
    if (use_dev) {
#ifdef WITH_CUDA_MEMORY
        cudaMalloc((void **)&u, N * 5 * sizeof(float));
        cudaMalloc((void **)&b, N * 3 * sizeof(float));
        cudaMalloc((void **)&uu, N * 5 * sizeof(float));
        cudaMalloc((void **)&ub, N * 3 * sizeof(float));
        cudaMemcpy(u, hu, N * 5 * sizeof(float), cudaMemcpyHostToDevice);
        cudaMemcpy(b, hb, N * 3 * sizeof(float), cudaMemcpyHostToDevice);
#else
        fprintf(stderr, "built without device memory support\n");
        return 2;
#endif
    } else {
        uu = malloc(N * 5 * sizeof(float));
        ub = malloc(N * 3 * sizeof(float));
    }
    /* both contexts start from the same state (C/mhd.c:50-51) */
    copy_matrix(u, b, &nx, &ny, &nz, uu, ub);

    float t = 0, tf = 1e30f, dt = 0;
    int iter = 0;
    do {
        iter = iter + 1;
        dt = cfl * calcfl(u, b, &nx, &ny, &nz);
        if (dt > (tf - t) / 2)
            dt = (tf - t) / 2;
        t = t + 2 * dt;
        fluidx(u, b, &nx, &ny, &nz, &dt, uu, ub, iter);
        copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        advectbyzx(u, b, &nx, &ny, &nz, &dt, uu, ub);
        copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        transpose12(u, b, uu, ub, &nx, &ny, &nz, iter);
        copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        fluidx(u, b, &ny, &nx, &nz, &dt, uu, ub, iter);
        copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        advectbyzx(u, b, &ny, &nx, &nz, &dt, uu, ub);
        copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        transpose13(u, b, uu, ub, &ny, &nx, &nz);
        copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        fluidx(u, b, &nz, &nx, &ny, &dt, uu, ub, iter);
        copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        advectbyzx(u, b, &nz, &nx, &ny, &dt, uu, ub);
        copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        advectbyzx(u, b, &nz, &nx, &ny, &dt, uu, ub);
        copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        fluidx(u, b, &nz, &nx, &ny, &dt, uu, ub, iter);
        copy_matrix(u, b, &nz, &nx, &ny, uu, ub);
        transpose13(u, b, uu, ub, &nz, &nx, &ny);
        copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        advectbyzx(u, b, &ny, &nx, &nz, &dt, uu, ub);
        copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        fluidx(u, b, &ny, &nx, &nz, &dt, uu, ub, iter);
        copy_matrix(u, b, &ny, &nx, &nz, uu, ub);
        transpose12(u, b, uu, ub, &ny, &nx, &nz, iter);
        copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        advectbyzx(u, b, &nx, &ny, &nz, &dt, uu, ub);
        copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
        fluidx(u, b, &nx, &ny, &nz, &dt, uu, ub, iter);
        copy_matrix(u, b, &nx, &ny, &nz, uu, ub);
    } while (iter < nsteps);

#ifdef WITH_CUDA_MEMORY
    if (use_dev) {
        cudaMemcpy(hu, u, N * 5 * sizeof(float), cudaMemcpyDeviceToHost);
        cudaMemcpy(hb, b, N * 3 * sizeof(float), cudaMemcpyDeviceToHost);
    }
#endif
    f = fopen(argv[2], "wb");
    fwrite(hu, sizeof(float), N * 5, f);
    fwrite(hb, sizeof(float), N * 3, f);
    fwrite(&t, sizeof(float), 1, f);
    fclose(f);
    return 0;
}
