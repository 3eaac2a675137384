/*
 * trackfile.c — the on-disk track format of include/moc_trackfile.h: CSR segment
 * descriptors with region and interval packed into one 32-bit cell index, lengths as FP32
 * (version 1, 8 bytes per segment) or IEEE half (version 2, 6 bytes per segment), a
 * 48-byte header and an FNV-1a checksum over the payload's 64-bit words. Host-only C, part
 * of libmocatt.so. The payload is streamed in chunks, so a file of any size needs only the
 * caller's arrays and one 1M-entry buffer.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "moc_trackfile.h"

static const char MAGIC[8] = {'M', 'O', 'C', 'T', 'R', 'K', '0', '1'};
enum { HEADER_BYTES = 48, VERSION_FP32 = 1, VERSION_HALF = 2, CHUNK = 1 << 20 };

/* IEEE binary32 -> binary16, rounded to nearest (ties to even), from the formats'
 * definitions: sign, 5-bit exponent (bias 15), 10-bit fraction; subnormals below 2^-14 in
 * units of 2^-24; values from 65520 on round to infinity. */
static uint16_t half_of(float x)
{
    uint32_t u;
    memcpy(&u, &x, 4);
    const uint32_t sign = (u >> 16) & 0x8000u, a = u & 0x7fffffffu;
    if (a >= 0x7f800000u) return (uint16_t)(sign | (a > 0x7f800000u ? 0x7e00u : 0x7c00u));
    if (a >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);
    if (a >= 0x38800000u) {  /* normal half */
        const uint32_t frac = a & 0x7fffffu, rem = frac & 0x1fffu;
        uint32_t h = (((a >> 23) - 112u) << 10) | (frac >> 13);
        if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) h++;
        return (uint16_t)(sign | h);
    }
    if (a < 0x33000000u) return (uint16_t)sign;  /* below 2^-25: zero */
    const uint32_t m = (a & 0x7fffffu) | 0x800000u;
    const int sh = 126 - (int)(a >> 23);  /* 14 .. 24 */
    uint32_t h = m >> sh;
    const uint32_t rem = m & ((1u << sh) - 1u), halfway = 1u << (sh - 1);
    if (rem > halfway || (rem == halfway && (h & 1u))) h++;
    return (uint16_t)(sign | h);
}

/* binary16 -> binary32, exact */
static float float_of(uint16_t h)
{
    const uint32_t sign = ((uint32_t)h & 0x8000u) << 16, e = (h >> 10) & 0x1fu, m = h & 0x3ffu;
    uint32_t u;
    if (e == 0) {
        const float v = (float)m * 5.9604644775390625e-8f;  /* m * 2^-24, exact */
        return sign ? -v : v;
    }
    if (e == 31) u = sign | 0x7f800000u | (m << 13);
    else u = sign | ((e + 112u) << 23) | (m << 13);
    float f;
    memcpy(&f, &u, 4);
    return f;
}

static int little_endian(void)
{
    const uint16_t x = 1;
    uint8_t b;
    memcpy(&b, &x, 1);
    return b == 1;
}

/* FNV-1a over little-endian 64-bit words, fed in pieces of any length */
typedef struct {
    uint64_t h;
    uint8_t part[8];
    int n;
} fnv_t;

static void fnv_word(fnv_t *f, uint64_t w) { f->h = (f->h ^ w) * 1099511628211ull; }

static void fnv_init(fnv_t *f)
{
    f->h = 14695981039346656037ull;
    f->n = 0;
}

static void fnv_bytes(fnv_t *f, const void *p, size_t len)
{
    const uint8_t *b = (const uint8_t *)p;
    while (len && f->n) {
        f->part[f->n++] = *b++;
        len--;
        if (f->n == 8) {
            uint64_t w;
            memcpy(&w, f->part, 8);
            fnv_word(f, w);
            f->n = 0;
        }
    }
    for (; len >= 8; b += 8, len -= 8) {
        uint64_t w;
        memcpy(&w, b, 8);
        fnv_word(f, w);
    }
    while (len--) f->part[f->n++] = *b++;
}

static uint64_t fnv_final(fnv_t *f)
{
    if (f->n) {
        memset(f->part + f->n, 0, (size_t)(8 - f->n));
        uint64_t w;
        memcpy(&w, f->part, 8);
        fnv_word(f, w);
        f->n = 0;
    }
    return f->h;
}

static void put_header(uint8_t *h, uint32_t version, int64_t T, int64_t S, int32_t R,
                       int32_t I, uint64_t sum)
{
    const uint32_t hbytes = HEADER_BYTES;
    memcpy(h, MAGIC, 8);
    memcpy(h + 8, &version, 4);
    memcpy(h + 12, &hbytes, 4);
    memcpy(h + 16, &T, 8);
    memcpy(h + 24, &S, 8);
    memcpy(h + 32, &R, 4);
    memcpy(h + 36, &I, 4);
    memcpy(h + 40, &sum, 8);
}

static moc_status_t write_file(const char *path, uint32_t version, int64_t T, int64_t S,
                               int32_t R, int32_t I, const int64_t *off, const int32_t *reg,
                               const uint8_t *itv, const float *ds)
{
    if (!little_endian()) return MOC_ERR_UNSUPPORTED;
    if (!path || T < 0 || S < 0 || R < 1 || I < 1 || (uint64_t)R * (uint64_t)I > 0xffffffffull ||
        !off || (S > 0 && (!reg || !itv || !ds)))
        return MOC_ERR_INVALID_ARG;
    if (off[0] != 0 || off[T] != S) return MOC_ERR_INVALID_ARG;
    for (int64_t t = 0; t < T; t++)
        if (off[t + 1] < off[t]) return MOC_ERR_INVALID_ARG;
    for (int64_t j = 0; j < S; j++)
        if ((uint32_t)reg[j] >= (uint32_t)R || itv[j] >= I) return MOC_ERR_INVALID_ARG;
    if (version == VERSION_HALF)
        for (int64_t j = 0; j < S; j++)  /* finite, >= 0, and finite as a half */
            if (!(ds[j] >= 0.0f) || (half_of(ds[j]) & 0x7c00u) == 0x7c00u)
                return MOC_ERR_INVALID_ARG;
    FILE *f = fopen(path, "wb");
    if (!f) return MOC_ERR_IO;
    uint32_t *buf = (uint32_t *)malloc((size_t)CHUNK * sizeof(uint32_t));
    uint8_t h[HEADER_BYTES];
    fnv_t sum;
    fnv_init(&sum);
    put_header(h, version, T, S, R, I, 0);
    int ok = buf && fwrite(h, 1, HEADER_BYTES, f) == HEADER_BYTES;
    ok = ok && fwrite(off, 8, (size_t)(T + 1), f) == (size_t)(T + 1);
    if (ok) fnv_bytes(&sum, off, (size_t)(T + 1) * 8);
    for (int64_t j0 = 0; ok && j0 < S; j0 += CHUNK) {
        const int64_t n = S - j0 < CHUNK ? S - j0 : CHUNK;
        for (int64_t j = 0; j < n; j++)
            buf[j] = (uint32_t)reg[j0 + j] * (uint32_t)I + (uint32_t)itv[j0 + j];
        ok = fwrite(buf, 4, (size_t)n, f) == (size_t)n;
        fnv_bytes(&sum, buf, (size_t)n * 4);
    }
    if (version == VERSION_FP32) {
        ok = ok && (S == 0 || fwrite(ds, 4, (size_t)S, f) == (size_t)S);
        if (ok) fnv_bytes(&sum, ds, (size_t)S * 4);
    } else {
        uint16_t *hb = (uint16_t *)buf;
        for (int64_t j0 = 0; ok && j0 < S; j0 += CHUNK) {
            const int64_t n = S - j0 < CHUNK ? S - j0 : CHUNK;
            for (int64_t j = 0; j < n; j++) hb[j] = half_of(ds[j0 + j]);
            ok = fwrite(hb, 2, (size_t)n, f) == (size_t)n;
            fnv_bytes(&sum, hb, (size_t)n * 2);
        }
    }
    if (ok) {
        put_header(h, version, T, S, R, I, fnv_final(&sum));
        ok = fseek(f, 0, SEEK_SET) == 0 && fwrite(h, 1, HEADER_BYTES, f) == HEADER_BYTES;
    }
    free(buf);
    if (fclose(f) != 0) ok = 0;
    return ok ? MOC_OK : MOC_ERR_IO;
}

moc_status_t moc_trackfile_write(const char *path, int64_t T, int64_t S, int32_t R, int32_t I,
                                 const int64_t *off, const int32_t *reg, const uint8_t *itv,
                                 const float *ds)
{
    return write_file(path, VERSION_FP32, T, S, R, I, off, reg, itv, ds);
}

moc_status_t moc_trackfile_write_compact(const char *path, int64_t T, int64_t S, int32_t R,
                                         int32_t I, const int64_t *off, const int32_t *reg,
                                         const uint8_t *itv, const float *ds)
{
    return write_file(path, VERSION_HALF, T, S, R, I, off, reg, itv, ds);
}

static moc_status_t read_header(FILE *f, moc_trackfile_info_t *info)
{
    uint8_t h[HEADER_BYTES];
    uint32_t version, hbytes;
    if (fread(h, 1, HEADER_BYTES, f) != HEADER_BYTES || memcmp(h, MAGIC, 8) != 0)
        return MOC_ERR_IO;
    memcpy(&version, h + 8, 4);
    memcpy(&hbytes, h + 12, 4);
    memcpy(&info->n_tracks, h + 16, 8);
    memcpy(&info->n_segments, h + 24, 8);
    memcpy(&info->n_regions, h + 32, 4);
    memcpy(&info->n_intervals, h + 36, 4);
    memcpy(&info->checksum, h + 40, 8);
    info->version = (int32_t)version;
    info->bytes_per_segment = version == VERSION_HALF ? 6 : 8;
    if ((version != VERSION_FP32 && version != VERSION_HALF) || hbytes != HEADER_BYTES ||
        info->n_tracks < 0 ||
        info->n_segments < 0 || info->n_regions < 1 || info->n_intervals < 1 ||
        info->n_tracks > ((int64_t)1 << 40) || info->n_segments > ((int64_t)1 << 40) ||
        (uint64_t)info->n_regions * (uint64_t)info->n_intervals > 0xffffffffull)
        return MOC_ERR_IO;
    return MOC_OK;
}

moc_status_t moc_trackfile_info(const char *path, moc_trackfile_info_t *info)
{
    if (!little_endian()) return MOC_ERR_UNSUPPORTED;
    if (!path || !info) return MOC_ERR_INVALID_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return MOC_ERR_IO;
    const moc_status_t s = read_header(f, info);
    fclose(f);
    return s;
}

moc_status_t moc_trackfile_read(const char *path, int64_t *off, int32_t *reg, uint8_t *itv,
                                float *ds)
{
    if (!little_endian()) return MOC_ERR_UNSUPPORTED;
    if (!path || !off) return MOC_ERR_INVALID_ARG;
    FILE *f = fopen(path, "rb");
    if (!f) return MOC_ERR_IO;
    moc_trackfile_info_t info;
    moc_status_t s = read_header(f, &info);
    const int64_t T = info.n_tracks, S = info.n_segments;
    const uint32_t I = (uint32_t)info.n_intervals;
    const uint64_t ncell = (uint64_t)info.n_regions * I;
    if (s == MOC_OK && S > 0 && (!reg || !itv || !ds)) s = MOC_ERR_INVALID_ARG;
    uint32_t *buf = s == MOC_OK ? (uint32_t *)malloc((size_t)CHUNK * sizeof(uint32_t)) : NULL;
    if (s == MOC_OK && !buf) s = MOC_ERR_IO;
    fnv_t sum;
    fnv_init(&sum);
    if (s == MOC_OK && fread(off, 8, (size_t)(T + 1), f) != (size_t)(T + 1)) s = MOC_ERR_IO;
    if (s == MOC_OK) fnv_bytes(&sum, off, (size_t)(T + 1) * 8);
    for (int64_t j0 = 0; s == MOC_OK && j0 < S; j0 += CHUNK) {
        const int64_t n = S - j0 < CHUNK ? S - j0 : CHUNK;
        if (fread(buf, 4, (size_t)n, f) != (size_t)n) {
            s = MOC_ERR_IO;
            break;
        }
        fnv_bytes(&sum, buf, (size_t)n * 4);
        for (int64_t j = 0; j < n; j++) {
            if (buf[j] >= ncell) {
                s = MOC_ERR_IO;
                break;
            }
            reg[j0 + j] = (int32_t)(buf[j] / I);
            itv[j0 + j] = (uint8_t)(buf[j] % I);
        }
    }
    if (info.version == VERSION_FP32) {
        if (s == MOC_OK && S > 0 && fread(ds, 4, (size_t)S, f) != (size_t)S) s = MOC_ERR_IO;
        if (s == MOC_OK) fnv_bytes(&sum, ds, (size_t)S * 4);
    } else {
        uint16_t *hb = (uint16_t *)buf;
        for (int64_t j0 = 0; s == MOC_OK && j0 < S; j0 += CHUNK) {
            const int64_t n = S - j0 < CHUNK ? S - j0 : CHUNK;
            if (fread(hb, 2, (size_t)n, f) != (size_t)n) {
                s = MOC_ERR_IO;
                break;
            }
            fnv_bytes(&sum, hb, (size_t)n * 2);
            for (int64_t j = 0; j < n; j++) ds[j0 + j] = float_of(hb[j]);
        }
    }
    if (s == MOC_OK && (fnv_final(&sum) != info.checksum || fgetc(f) != EOF)) s = MOC_ERR_IO;
    if (s == MOC_OK) {
        if (off[0] != 0 || off[T] != S) s = MOC_ERR_IO;
        for (int64_t t = 0; s == MOC_OK && t < T; t++)
            if (off[t + 1] < off[t]) s = MOC_ERR_IO;
    }
    free(buf);
    fclose(f);
    return s;
}
