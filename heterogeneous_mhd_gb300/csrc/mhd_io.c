/* File formats around the state (host arrays): the reference's check_value
 * text dump and init reader, and a binary checkpoint.
 *
 * The state layout is the reference's: u(5,nx,ny,nz), b(3,nx,ny,nz),
 * component index fastest, then i, j, k (C/array_definition.h:12).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mhd_io.h"

static double getv(const void *a, int fp64, size_t i)
{
    return fp64 ? ((const double *)a)[i] : (double)((const float *)a)[i];
}

static void putv(void *a, int fp64, size_t i, double v)
{
    if (fp64)
        ((double *)a)[i] = v;
    else
        ((float *)a)[i] = (float)v;
}

/* C/check_value.c:25-66: eight files C_version_check_{u1..u5,b1..b3}.dat in
 * `dir`, one "%8.6e" value per line, i fastest, then j, then k. */
MHD_API int mhd_write_check_value(const void *u, const void *b, int nx, int ny, int nz, int fp64, const char *dir)
{
    if (!u || !b || nx <= 0 || ny <= 0 || nz <= 0)
        return MHD_ERR_ARG;
    static const char *names[8] = {"u1", "u2", "u3", "u4", "u5", "b1", "b2", "b3"};
    FILE *f[8] = {0};
    char path[4096];
    int st = MHD_OK;
    for (int q = 0; q < 8 && st == MHD_OK; q++) {
        snprintf(path, sizeof(path), "%s%sC_version_check_%s.dat", dir ? dir : "", (dir && *dir) ? "/" : "", names[q]);
        f[q] = fopen(path, "w");
        if (!f[q])
            st = MHD_ERR_ARG;
    }
    const size_t cells = (size_t)nx * ny * nz;
    for (size_t c = 0; c < cells && st == MHD_OK; c++) { /* c = i + nx (j + ny k): the i-fastest order */
        for (int q = 0; q < 5; q++)
            fprintf(f[q], "%8.6e\n", getv(u, fp64, 5 * c + q));
        for (int q = 0; q < 3; q++)
            fprintf(f[5 + q], "%8.6e\n", getv(b, fp64, 3 * c + q));
    }
    for (int q = 0; q < 8; q++)
        if (f[q] && fclose(f[q]) != 0)
            st = MHD_ERR_ARG;
    return st;
}

/* C/init.c:34-52: 8 whitespace-separated values per cell (u1..u5, b1..b3),
 * cells in i-outer, j, k-inner order. */
MHD_API int mhd_read_init(const char *path, void *u, void *b, int nx, int ny, int nz, int fp64)
{
    if (!path || !u || !b || nx <= 0 || ny <= 0 || nz <= 0)
        return MHD_ERR_ARG;
    FILE *f = fopen(path, "r");
    if (!f)
        return MHD_ERR_ARG;
    int st = MHD_OK;
    for (int i = 0; i < nx && st == MHD_OK; i++)
        for (int j = 0; j < ny && st == MHD_OK; j++)
            for (int k = 0; k < nz && st == MHD_OK; k++) {
                const size_t c = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * (size_t)k);
                for (int q = 0; q < 8; q++) {
                    float v;
                    if (fscanf(f, "%f", &v) != 1) {
                        st = MHD_ERR_ARG;
                        break;
                    }
                    if (q < 5)
                        putv(u, fp64, 5 * c + q, v);
                    else
                        putv(b, fp64, 3 * c + (q - 5), v);
                }
            }
    fclose(f);
    return st;
}

/* ---------------------------------------------------------- checkpoints */

/* header (64 bytes, little-endian): "MHDGB300", u32 version, u32 element
 * size, i32 nx ny nz, u32 0, f64 t, i64 step, u64 FNV-1a of the payload,
 * 8 bytes 0; then u and b as stored in memory */
struct ckpt_header {
    char magic[8];
    uint32_t version, elem;
    int32_t nx, ny, nz;
    uint32_t pad;
    double t;
    int64_t step;
    uint64_t hash;
    uint64_t pad2;
};

static uint64_t fnv1a(uint64_t h, const void *p, size_t n)
{
    const unsigned char *s = (const unsigned char *)p;
    for (size_t i = 0; i < n; i++) {
        h ^= s[i];
        h *= 0x100000001b3ULL;
    }
    return h;
}

MHD_API int mhd_checkpoint_save(const char *path, const void *u, const void *b, int nx, int ny, int nz, int fp64,
                                double t, long long step)
{
    if (!path || !u || !b || nx <= 0 || ny <= 0 || nz <= 0)
        return MHD_ERR_ARG;
    const size_t cells = (size_t)nx * ny * nz, es = fp64 ? 8 : 4;
    struct ckpt_header h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "MHDGB300", 8);
    h.version = 1;
    h.elem = (uint32_t)es;
    h.nx = nx, h.ny = ny, h.nz = nz;
    h.t = t;
    h.step = step;
    h.hash = fnv1a(fnv1a(0xcbf29ce484222325ULL, u, 5 * cells * es), b, 3 * cells * es);
    FILE *f = fopen(path, "wb");
    if (!f)
        return MHD_ERR_ARG;
    int ok = fwrite(&h, sizeof(h), 1, f) == 1 && fwrite(u, es, 5 * cells, f) == 5 * cells &&
             fwrite(b, es, 3 * cells, f) == 3 * cells;
    ok = (fclose(f) == 0) && ok;
    return ok ? MHD_OK : MHD_ERR_ARG;
}

MHD_API int mhd_checkpoint_info(const char *path, int *nx, int *ny, int *nz, int *fp64, double *t, long long *step)
{
    if (!path)
        return MHD_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f)
        return MHD_ERR_ARG;
    struct ckpt_header h;
    const int ok = fread(&h, sizeof(h), 1, f) == 1;
    fclose(f);
    if (!ok || memcmp(h.magic, "MHDGB300", 8) != 0 || h.version != 1 || (h.elem != 4 && h.elem != 8))
        return MHD_ERR_ARG;
    if (nx) *nx = h.nx;
    if (ny) *ny = h.ny;
    if (nz) *nz = h.nz;
    if (fp64) *fp64 = h.elem == 8;
    if (t) *t = h.t;
    if (step) *step = h.step;
    return MHD_OK;
}

MHD_API int mhd_checkpoint_load(const char *path, void *u, void *b, int nx, int ny, int nz, int fp64, double *t,
                                long long *step)
{
    if (!path || !u || !b)
        return MHD_ERR_ARG;
    FILE *f = fopen(path, "rb");
    if (!f)
        return MHD_ERR_ARG;
    struct ckpt_header h;
    const size_t cells = (size_t)nx * ny * nz, es = fp64 ? 8 : 4;
    int ok = fread(&h, sizeof(h), 1, f) == 1 && memcmp(h.magic, "MHDGB300", 8) == 0 && h.version == 1 &&
             h.elem == es && h.nx == nx && h.ny == ny && h.nz == nz;
    ok = ok && fread(u, es, 5 * cells, f) == 5 * cells && fread(b, es, 3 * cells, f) == 3 * cells;
    char extra;
    ok = ok && fread(&extra, 1, 1, f) == 0; /* nothing after the payload */
    fclose(f);
    if (!ok || fnv1a(fnv1a(0xcbf29ce484222325ULL, u, 5 * cells * es), b, 3 * cells * es) != h.hash)
        return MHD_ERR_ARG;
    if (t) *t = h.t;
    if (step) *step = h.step;
    return MHD_OK;
}
