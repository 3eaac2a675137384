/*
 * trackfile.c — the oracle's reader of the on-disk track format (include/moc_trackfile.h).
 *
 * TEST AND BENCH INFRASTRUCTURE ONLY: lets the CPU harness (cpu_bench --track-file) sweep
 * the same segment files as the GPU program (mocatt_run -f). Restated from the header's
 * layout, independently of the library's reader (simplemoc-kernel_gb300/host/trackfile.c).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* IEEE half -> float, exact: 5-bit exponent (bias 15), 10-bit fraction, subnormals in
 * units of 2^-24. */
static float half_to_float(uint16_t h)
{
    const int e = (h >> 10) & 31, m = h & 1023;
    const float sign = (h & 0x8000) ? -1.0f : 1.0f;
    if (e == 0) return sign * ldexpf((float)m, -24);
    if (e == 31) return m ? NAN : sign * INFINITY;
    return sign * ldexpf((float)(1024 + m), e - 25);
}

static uint64_t fnv_update(uint64_t h, const uint8_t *p, size_t n, uint8_t *carry, int *nc)
{
    for (size_t i = 0; i < n; i++) {
        carry[(*nc)++] = p[i];
        if (*nc == 8) {
            uint64_t w = 0;
            for (int b = 7; b >= 0; b--) w = (w << 8) | carry[b];
            h = (h ^ w) * 1099511628211ull;
            *nc = 0;
        }
    }
    return h;
}

int oracle_trackfile_read(const char *path, int64_t *T_out, int64_t *S_out, int32_t *R_out,
                          int32_t *I_out, int64_t **off, int32_t **reg, uint8_t **itv,
                          float **ds)
{
    FILE *f = fopen(path, "rb");
    if (!f) return -1;
    uint8_t h[48];
    int64_t T, S;
    int32_t R, I;
    uint32_t version, hbytes;
    uint64_t sum;
    if (fread(h, 1, 48, f) != 48 || memcmp(h, "MOCTRK01", 8) != 0) {
        fclose(f);
        return -1;
    }
    memcpy(&version, h + 8, 4);
    memcpy(&hbytes, h + 12, 4);
    memcpy(&T, h + 16, 8);
    memcpy(&S, h + 24, 8);
    memcpy(&R, h + 32, 4);
    memcpy(&I, h + 36, 4);
    memcpy(&sum, h + 40, 8);
    if ((version != 1 && version != 2) || hbytes != 48 || T < 0 || S < 0 || R < 1 || I < 1) {
        fclose(f);
        return -1;
    }
    const int per = version == 1 ? 8 : 6;  /* bytes per segment: cell + length */
    const size_t n = (size_t)(8 * (T + 1) + per * S);
    uint8_t *payload = (uint8_t *)malloc(n ? n : 1);
    if (!payload || fread(payload, 1, n, f) != n || fgetc(f) != EOF) {
        free(payload);
        fclose(f);
        return -1;
    }
    fclose(f);
    uint8_t carry[8];
    int nc = 0;
    uint64_t hsh = fnv_update(14695981039346656037ull, payload, n, carry, &nc);
    if (nc) {  /* the last word, zero-padded */
        memset(carry + nc, 0, (size_t)(8 - nc));
        uint64_t w = 0;
        for (int b = 7; b >= 0; b--) w = (w << 8) | carry[b];
        hsh = (hsh ^ w) * 1099511628211ull;
    }
    *off = (int64_t *)malloc((size_t)(T + 1) * 8);
    *reg = (int32_t *)malloc((size_t)(S ? S : 1) * 4);
    *itv = (uint8_t *)malloc((size_t)(S ? S : 1));
    *ds = (float *)malloc((size_t)(S ? S : 1) * 4);
    int ok = hsh == sum && *off && *reg && *itv && *ds;
    if (ok) {
        memcpy(*off, payload, (size_t)(T + 1) * 8);
        ok = (*off)[0] == 0 && (*off)[T] == S;
        for (int64_t t = 0; ok && t < T; t++) ok = (*off)[t + 1] >= (*off)[t];
        for (int64_t j = 0; ok && j < S; j++) {
            uint32_t c;
            memcpy(&c, payload + 8 * (T + 1) + 4 * j, 4);
            ok = c < (uint64_t)R * (uint64_t)I;
            (*reg)[j] = (int32_t)(c / (uint32_t)I);
            (*itv)[j] = (uint8_t)(c % (uint32_t)I);
        }
        if (ok && version == 1) memcpy(*ds, payload + 8 * (T + 1) + 4 * S, (size_t)S * 4);
        for (int64_t j = 0; ok && version == 2 && j < S; j++) {
            uint16_t hv;
            memcpy(&hv, payload + 8 * (T + 1) + 4 * S + 2 * j, 2);
            (*ds)[j] = half_to_float(hv);
        }
    }
    free(payload);
    if (!ok) {
        free(*off);
        free(*reg);
        free(*itv);
        free(*ds);
        *off = NULL;
        *reg = NULL;
        *itv = NULL;
        *ds = NULL;
        return -1;
    }
    *T_out = T;
    *S_out = S;
    *R_out = R;
    *I_out = I;
    return 0;
}
