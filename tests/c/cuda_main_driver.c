/*
 * A time-stepping driver written only against the reference's CUDA-side call
 * surface (Cuda/cuda_subroutine.h:4-12): it replays the loop of
 * Cuda/cuda_main.cu:72-116 on cudaMalloc arrays, with the reference's
 * device and host copies of the dimensions, its `temp` EMF scratch and its
 * `c` CFL scratch, and links against libmhd_gb300.so through
 * include/mhd_cuda_compat.h.
 *
 * One departure from the reference's loop, so that the time step is the C
 * path's (C/mhd.c:62-64): Cuda/cuda_cfl.cu:41-43 leaves 1/c in the device dt
 * and Cuda/cuda_main.cu:84-86 computes dt = cfl/c and its clamp on the host
 * only, so the reference's sweeps never see the CFL factor; here the host dt
 * is copied to the device before the sweeps.
 *
 * usage: cuda_main_driver in.bin out.bin nx ny nz nsteps cfl
 *   in.bin : u (5*N floats) then b (3*N floats), N = nx*ny*nz
 *   out.bin: u, b after nsteps, then t (1 float)
 * Exit status 0, or 1 with a message when a call records an error.
 */
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime.h>

#include "mhd_cuda_compat.h"

static int check(const char *what)
{
    const int s = mhd_last_error();
    if (s != MHD_OK) {
        fprintf(stderr, "%s: %s\n", what, mhd_error_string(s));
        return 1;
    }
    return 0;
}

#define CALL(x)              \
    do {                     \
        x;                   \
        if (check(#x))       \
            return 1;        \
    } while (0)

int main(int argc, char **argv)
{
    if (argc < 8) {
        fprintf(stderr, "usage: %s in.bin out.bin nx ny nz nsteps cfl\n", argv[0]);
        return 2;
    }
    int h_dims[3] = {atoi(argv[3]), atoi(argv[4]), atoi(argv[5])};
    int *h_nx = &h_dims[0], *h_ny = &h_dims[1], *h_nz = &h_dims[2];
    const int nsteps = atoi(argv[6]);
    const double cfl = atof(argv[7]);
    const size_t N = (size_t)(*h_nx) * (*h_ny) * (*h_nz);
    const size_t u_mem = 5 * N * sizeof(float), b_mem = 3 * N * sizeof(float);
    float *h_u = malloc(u_mem), *h_b = malloc(b_mem);
    FILE *f = fopen(argv[1], "rb");
    if (!f || fread(h_u, 1, u_mem, f) != u_mem || fread(h_b, 1, b_mem, f) != b_mem) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 1;
    }
    fclose(f);

    /* device state, transpose targets, scratch and dimension copies, as
     * Cuda/cuda_main.cu:31-55 sets them up */
    float *d_u, *d_b, *d_ut, *d_bt, *d_dt, *d_c, *d_temp;
    int *d_nx, *d_ny, *d_nz;
    if (cudaMalloc((void **)&d_u, u_mem) != cudaSuccess || cudaMalloc((void **)&d_b, b_mem) != cudaSuccess ||
        cudaMalloc((void **)&d_ut, u_mem) != cudaSuccess || cudaMalloc((void **)&d_bt, b_mem) != cudaSuccess ||
        cudaMalloc((void **)&d_dt, sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&d_c, (size_t)(*h_ny) * (*h_nz) * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&d_temp, N * sizeof(float)) != cudaSuccess ||
        cudaMalloc((void **)&d_nx, sizeof(int)) != cudaSuccess || cudaMalloc((void **)&d_ny, sizeof(int)) != cudaSuccess ||
        cudaMalloc((void **)&d_nz, sizeof(int)) != cudaSuccess) {
        fprintf(stderr, "cudaMalloc failed\n");
        return 1;
    }
    cudaMemcpy(d_u, h_u, u_mem, cudaMemcpyHostToDevice);
    cudaMemcpy(d_b, h_b, b_mem, cudaMemcpyHostToDevice);
    cudaMemcpy(d_nx, h_nx, sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_ny, h_ny, sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(d_nz, h_nz, sizeof(int), cudaMemcpyHostToDevice);

    float t = 0, tf = 1e30f, dt = 0, h_dt = 0;
    int iter = 0;
    do {
        iter = iter + 1;
        CALL(cuda_cfl(d_u, d_b, d_nx, d_ny, d_nz, d_dt, d_c, h_nx, h_ny, h_nz, &h_dt));
        dt = cfl * h_dt;
        if (dt > (tf - t) / 2) /* C/mhd.c:63 */
            dt = (tf - t) / 2;
        t = t + 2 * dt;
        cudaMemcpy(d_dt, &dt, sizeof(float), cudaMemcpyHostToDevice);
        /* x sweep */
        CALL(cuda_fluidx(d_u, d_b, d_nx, d_ny, d_nz, d_dt, h_nx, h_ny, h_nz));
        CALL(cuda_advectbyzx(d_u, d_b, d_nx, d_ny, d_nz, d_dt, d_temp, h_nx, h_ny, h_nz));
        /* y sweep */
        CALL(cuda_transpose12(d_ut, d_bt, d_u, d_b, d_nx, d_ny, d_nz, h_nx, h_ny, h_nz));
        CALL(cuda_fluidx(d_u, d_b, d_ny, d_nx, d_nz, d_dt, h_ny, h_nx, h_nz));
        CALL(cuda_advectbyzx(d_u, d_b, d_ny, d_nx, d_nz, d_dt, d_temp, h_ny, h_nx, h_nz));
        /* z sweep */
        CALL(cuda_transpose13(d_ut, d_bt, d_u, d_b, d_ny, d_nx, d_nz, h_ny, h_nx, h_nz));
        CALL(cuda_fluidx(d_u, d_b, d_nz, d_nx, d_ny, d_dt, h_nz, h_nx, h_ny));
        CALL(cuda_advectbyzx(d_u, d_b, d_nz, d_nx, d_ny, d_dt, d_temp, h_nz, h_nx, h_ny));
        CALL(cuda_advectbyzx(d_u, d_b, d_nz, d_nx, d_ny, d_dt, d_temp, h_nz, h_nx, h_ny));
        CALL(cuda_fluidx(d_u, d_b, d_nz, d_nx, d_ny, d_dt, h_nz, h_nx, h_ny));
        /* back */
        CALL(cuda_transpose13(d_ut, d_bt, d_u, d_b, d_nz, d_nx, d_ny, h_nz, h_nx, h_ny));
        CALL(cuda_advectbyzx(d_u, d_b, d_ny, d_nx, d_nz, d_dt, d_temp, h_ny, h_nx, h_nz));
        CALL(cuda_fluidx(d_u, d_b, d_ny, d_nx, d_nz, d_dt, h_ny, h_nx, h_nz));
        /* x again */
        CALL(cuda_transpose12(d_ut, d_bt, d_u, d_b, d_ny, d_nx, d_nz, h_ny, h_nx, h_nz));
        CALL(cuda_advectbyzx(d_u, d_b, d_nx, d_ny, d_nz, d_dt, d_temp, h_nx, h_ny, h_nz));
        CALL(cuda_fluidx(d_u, d_b, d_nx, d_ny, d_nz, d_dt, h_nx, h_ny, h_nz));
    } while (t < tf && iter < nsteps);

    if (cudaMemcpy(h_u, d_u, u_mem, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(h_b, d_b, b_mem, cudaMemcpyDeviceToHost) != cudaSuccess) {
        fprintf(stderr, "copy-out failed\n");
        return 1;
    }
    f = fopen(argv[2], "wb");
    if (!f) {
        fprintf(stderr, "cannot write %s\n", argv[2]);
        return 1;
    }
    fwrite(h_u, 1, u_mem, f);
    fwrite(h_b, 1, b_mem, f);
    fwrite(&t, sizeof(float), 1, f);
    fclose(f);
    return 0;
}
