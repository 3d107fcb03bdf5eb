/* cmcg_h5.c -- the CMC initial-conditions file (COSMIC's InitialCMCTable
 * output, an HDF5 file in pandas' fixed format) without the HDF5 library.
 *
 * Replaces cmc_read_hdf5_file (src/libs/fitslib.c:209-455), which opens the
 * datasets CLUS_OBJ_DATA/block0_values (one row per object: id, k, m, Reff,
 * r, vr, vt, binind) and CLUS_BINARY_DATA/block0_values (one row per binary:
 * index, id1, k1, m1, Reff1, id2, k2, m2, Reff2, a, e) as 2-D float64
 * arrays, and the scalar attributes NOBJ, NBINARY, MCLUS, RVIR, RTID and Z
 * of the first.  This reader walks the file's own structures as the HDF5
 * file-format specification (version 0 superblock) lays them out:
 *   superblock -> root group's symbol-table entry -> v1 B-tree of the group
 *   (type 0 nodes) -> symbol-table nodes -> names in the group's local heap
 *   -> version 1 object headers (with continuation blocks) -> dataspace,
 *   datatype, data-layout and attribute messages.
 * It reads what that file holds: contiguous (or compact) little-endian
 * float64 datasets, and float64 / int64 scalar attributes.  Anything else --
 * chunked or filtered storage, big-endian or other number types, a later
 * superblock -- is refused with an error, never guessed at.  Every offset is
 * checked against the file's length before it is followed. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cmcgpu.h"

enum { H5_MAX_MSGS = 4096, H5_MAX_DEPTH = 16 };

typedef struct {
    const unsigned char *d;
    size_t n;
} H5File;

typedef struct {
    int rank;
    uint64_t dims[8];
    int dtype_class, dtype_size, dtype_signed;  /* class 0 fixed-point, 1 floating-point */
    int layout;                                 /* 0 compact, 1 contiguous, -1 none */
    uint64_t data_addr, data_size;
    const unsigned char *compact;               /* compact layout: the data in the header */
    int filtered;
} H5Dataset;

static int rd(const H5File *f, uint64_t off, uint64_t len)
{
    return off <= f->n && len <= f->n - off;
}

static uint64_t le(const unsigned char *p, int n)
{
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

/* ---- groups: name -> object header address ------------------------------ */

/* the null-terminated name at offset `off` of the local heap at `heap` */
static const char *heap_name(const H5File *f, uint64_t heap, uint64_t off)
{
    if (!rd(f, heap, 32) || memcmp(f->d + heap, "HEAP", 4)) return NULL;
    const uint64_t size = le(f->d + heap + 8, 8), data = le(f->d + heap + 24, 8);
    if (off >= size || !rd(f, data, size)) return NULL;
    const char *s = (const char *)f->d + data + off;
    if (!memchr(s, 0, size - off)) return NULL;
    return s;
}

/* Object header address of `name` in the group whose v1 B-tree is at `btree`
 * and local heap at `heap`; 0 if absent or malformed. */
static uint64_t group_find(const H5File *f, uint64_t btree, uint64_t heap, const char *name, int depth)
{
    if (depth > H5_MAX_DEPTH || !rd(f, btree, 24) || memcmp(f->d + btree, "TREE", 4)) return 0;
    const unsigned char *p = f->d + btree;
    if (p[4] != 0) return 0;  /* node type 0: group nodes */
    const int level = p[5], used = (int)le(p + 6, 2);
    /* keys (8-byte heap offsets) and children (8-byte addresses) alternate, key first */
    if (!rd(f, btree + 24, (uint64_t)(2 * used + 1) * 8)) return 0;
    for (int i = 0; i < used; ++i) {
        const uint64_t child = le(p + 24 + (uint64_t)(2 * i + 1) * 8, 8);
        if (level > 0) {
            const uint64_t a = group_find(f, child, heap, name, depth + 1);
            if (a) return a;
            continue;
        }
        if (!rd(f, child, 8) || memcmp(f->d + child, "SNOD", 4)) return 0;
        const int nsym = (int)le(f->d + child + 6, 2);
        if (!rd(f, child + 8, (uint64_t)nsym * 40)) return 0;
        for (int s = 0; s < nsym; ++s) {
            const unsigned char *e = f->d + child + 8 + (uint64_t)s * 40;
            const char *nm = heap_name(f, heap, le(e, 8));
            if (nm && !strcmp(nm, name)) return le(e + 8, 8);
        }
    }
    return 0;
}

/* ---- object headers ------------------------------------------------------ */

typedef struct {
    int type;
    const unsigned char *data;
    uint64_t size;
} H5Msg;

/* The messages of the version 1 object header at `oh`, following
 * continuation messages; returns their number, -1 if malformed. */
static int header_messages(const H5File *f, uint64_t oh, H5Msg *out, int cap)
{
    if (!rd(f, oh, 16) || f->d[oh] != 1) return -1;
    const int total = (int)le(f->d + oh + 2, 2);
    uint64_t blk = oh + 16, len = le(f->d + oh + 8, 4);
    uint64_t conts[H5_MAX_DEPTH][2];
    int ncont = 0, n = 0, seen = 0;
    for (;;) {
        if (!rd(f, blk, len)) return -1;
        uint64_t q = 0;
        while (q + 8 <= len && seen < total) {
            const unsigned char *h = f->d + blk + q;
            const int type = (int)le(h, 2);
            const uint64_t size = le(h + 2, 2);
            if (q + 8 + size > len) return -1;
            ++seen;
            if (type == 0x10) {  /* continuation: another block of messages */
                if (size < 16 || ncont == H5_MAX_DEPTH) return -1;
                conts[ncont][0] = le(h + 8, 8);
                conts[ncont][1] = le(h + 16, 8);
                ++ncont;
            } else if (n < cap) {
                out[n].type = type;
                out[n].data = h + 8;
                out[n].size = size;
                ++n;
            }
            q += 8 + size;
        }
        if (seen >= total || ncont == 0) break;
        --ncont;
        blk = conts[ncont][0];
        len = conts[ncont][1];
    }
    return n;
}

static int parse_dataspace(const unsigned char *p, uint64_t size, H5Dataset *ds)
{
    if (size < 8) return -1;
    const int ver = p[0], rank = p[1];
    if (rank > 8) return -1;
    uint64_t off;
    if (ver == 1) {
        off = 8;
    } else if (ver == 2) {
        if (p[3] == 2) return -1;  /* null dataspace */
        off = 4;
    } else {
        return -1;
    }
    if (off + (uint64_t)rank * 8 > size) return -1;
    ds->rank = rank;
    for (int i = 0; i < rank; ++i) ds->dims[i] = le(p + off + 8 * (uint64_t)i, 8);
    return 0;
}

static int parse_datatype(const unsigned char *p, uint64_t size, H5Dataset *ds)
{
    if (size < 8) return -1;
    ds->dtype_class = p[0] & 0x0f;
    ds->dtype_size = (int)le(p + 4, 4);
    if (p[1] & 1) return -1;  /* big-endian */
    ds->dtype_signed = (p[1] >> 3) & 1;
    return 0;
}

static int parse_layout(const H5File *f, const unsigned char *p, uint64_t size, H5Dataset *ds)
{
    if (size < 2) return -1;
    const int ver = p[0];
    if (ver == 3) {
        const int cls = p[1];
        if (cls == 0) {  /* compact: size (2) + data */
            if (size < 4) return -1;
            ds->layout = 0;
            ds->data_size = le(p + 2, 2);
            if (4 + ds->data_size > size) return -1;
            ds->compact = p + 4;
            return 0;
        }
        if (cls == 1) {  /* contiguous: address (8) + size (8) */
            if (size < 18) return -1;
            ds->layout = 1;
            ds->data_addr = le(p + 2, 8);
            ds->data_size = le(p + 10, 8);
            return rd(f, ds->data_addr, ds->data_size) ? 0 : -1;
        }
        return -1;  /* chunked or virtual storage */
    }
    if (ver == 1 || ver == 2) {
        const int nd = p[1], cls = p[2];
        if (cls != 1 || size < 16 + 4 * (uint64_t)nd) return -1;
        ds->layout = 1;
        ds->data_addr = le(p + 8, 8);
        uint64_t elems = 1;
        for (int i = 0; i < nd; ++i) elems *= le(p + 16 + 4 * i, 4);
        ds->data_size = elems;  /* in elements here; the caller checks against the dataspace */
        return rd(f, ds->data_addr, 1) ? 0 : -1;
    }
    return -1;
}

/* Dataset `name` under the root group's subgroup `group`. */
static int open_dataset(const H5File *f, const char *group, const char *name, H5Dataset *ds, uint64_t *oh_out)
{
    memset(ds, 0, sizeof(*ds));
    ds->layout = -1;
    if (f->n < 96 || memcmp(f->d, "\x89HDF\r\n\x1a\n", 8)) return CMCG_ERR_FORMAT;
    if (f->d[8] != 0 || f->d[13] != 8 || f->d[14] != 8) return CMCG_ERR_FORMAT;  /* v0, 8-byte offsets */
    /* root group symbol-table entry at 56: cache type 1 holds its B-tree and heap */
    if (le(f->d + 56 + 16, 4) != 1) return CMCG_ERR_FORMAT;
    const uint64_t rbt = le(f->d + 56 + 24, 8), rheap = le(f->d + 56 + 32, 8);
    const uint64_t goh = group_find(f, rbt, rheap, group, 0);
    if (!goh) return CMCG_ERR_FORMAT;
    /* the subgroup's symbol-table message (0x11): its B-tree and heap */
    H5Msg m[64];
    int nm = header_messages(f, goh, m, 64);
    uint64_t gbt = 0, gheap = 0;
    for (int i = 0; i < nm; ++i)
        if (m[i].type == 0x11 && m[i].size >= 16) {
            gbt = le(m[i].data, 8);
            gheap = le(m[i].data + 8, 8);
        }
    if (!gbt) return CMCG_ERR_FORMAT;
    const uint64_t doh = group_find(f, gbt, gheap, name, 0);
    if (!doh) return CMCG_ERR_FORMAT;
    *oh_out = doh;
    H5Msg *dm = (H5Msg *)malloc(sizeof(H5Msg) * H5_MAX_MSGS);
    if (!dm) return CMCG_ERR_NOMEM;
    nm = header_messages(f, doh, dm, H5_MAX_MSGS);
    int rc = nm < 0 ? CMCG_ERR_FORMAT : CMCG_OK;
    for (int i = 0; i < nm && rc == CMCG_OK; ++i) {
        if (dm[i].type == 0x01 && parse_dataspace(dm[i].data, dm[i].size, ds)) rc = CMCG_ERR_FORMAT;
        if (dm[i].type == 0x03 && parse_datatype(dm[i].data, dm[i].size, ds)) rc = CMCG_ERR_FORMAT;
        if (dm[i].type == 0x08 && parse_layout(f, dm[i].data, dm[i].size, ds)) rc = CMCG_ERR_FORMAT;
        if (dm[i].type == 0x0b) ds->filtered = 1;
    }
    free(dm);
    if (rc) return rc;
    if (ds->filtered || ds->layout < 0 || ds->rank != 2) return CMCG_ERR_FORMAT;
    if (ds->dtype_class != 1 || ds->dtype_size != 8) return CMCG_ERR_FORMAT;  /* float64 */
    const uint64_t elems = ds->dims[0] * ds->dims[1];
    if (ds->dims[1] && elems / ds->dims[1] != ds->dims[0]) return CMCG_ERR_FORMAT;
    const uint64_t bytes = elems * 8;
    if (ds->layout == 1 && ds->data_size != bytes && ds->data_size != elems) return CMCG_ERR_FORMAT;
    if (ds->layout == 0 && ds->data_size != bytes) return CMCG_ERR_FORMAT;
    if (ds->layout == 1 && !rd(f, ds->data_addr, bytes)) return CMCG_ERR_FORMAT;
    return CMCG_OK;
}

/* Scalar numeric attribute `name` of the object header at `oh` as a double
 * (float64 or 64-bit integer storage). */
static int attribute(const H5File *f, uint64_t oh, const char *name, double *out)
{
    H5Msg *m = (H5Msg *)malloc(sizeof(H5Msg) * H5_MAX_MSGS);
    if (!m) return CMCG_ERR_NOMEM;
    const int nm = header_messages(f, oh, m, H5_MAX_MSGS);
    int rc = CMCG_ERR_FORMAT;
    for (int i = 0; i < nm; ++i) {
        if (m[i].type != 0x0c) continue;
        const unsigned char *p = m[i].data;
        const uint64_t size = m[i].size;
        if (size < 8) break;
        const int ver = p[0];
        const uint64_t nlen = le(p + 2, 2), tlen = le(p + 4, 2), slen = le(p + 6, 2);
        uint64_t o = 8;
        if (ver == 3) o = 9;
        else if (ver != 1 && ver != 2) continue;
        const uint64_t pad = ver == 1 ? 8 : 1;
#define ALIGN(x) (((x) + pad - 1) / pad * pad)
        const uint64_t name_at = o, type_at = name_at + ALIGN(nlen), space_at = type_at + ALIGN(tlen),
                       data_at = space_at + ALIGN(slen);
#undef ALIGN
        if (data_at > size || nlen == 0) continue;
        /* the stored name (nlen bytes, its terminator included) equals `name` */
        const size_t want = strlen(name);
        if (nlen != want + 1 || memcmp(p + name_at, name, want) || p[name_at + want] != 0) continue;
        H5Dataset t;
        memset(&t, 0, sizeof(t));
        if (tlen < 8 || parse_datatype(p + type_at, tlen, &t) || t.dtype_size != 8) break;
        if (slen >= 8) {  /* scalar, or a one-element simple dataspace */
            H5Dataset s;
            memset(&s, 0, sizeof(s));
            if (parse_dataspace(p + space_at, slen, &s)) break;
            uint64_t elems = 1;
            for (int d = 0; d < s.rank; ++d) elems *= s.dims[d];
            if (elems != 1) break;
        }
        if (data_at + 8 > size) break;
        const uint64_t bits = le(p + data_at, 8);
        if (t.dtype_class == 1) {
            double v;
            memcpy(&v, &bits, 8);
            *out = v;
        } else if (t.dtype_class == 0) {
            *out = t.dtype_signed ? (double)(int64_t)bits : (double)bits;
        } else {
            break;
        }
        rc = CMCG_OK;
        break;
    }
    free(m);
    return rc;
}

static int copy_table(const H5File *f, const H5Dataset *ds, double *dst, long cap_rows)
{
    if (!dst) return CMCG_OK;
    if ((uint64_t)cap_rows < ds->dims[0]) return CMCG_ERR_CAPACITY;
    const unsigned char *src = ds->layout == 0 ? ds->compact : f->d + ds->data_addr;
    const uint64_t n = ds->dims[0] * ds->dims[1];
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t bits = le(src + 8 * i, 8);
        memcpy(dst + i, &bits, 8);
    }
    return CMCG_OK;
}

int cmcg_read_cmc_hdf5(const char *path, cmcg_cmc_hdf5_info *info, double *obj, long obj_cap_rows, double *bin,
                       long bin_cap_rows)
{
    if (!path || !info) return CMCG_ERR_ARG;
    memset(info, 0, sizeof(*info));
    FILE *fp = fopen(path, "rb");
    if (!fp) return CMCG_ERR_IO;
    int rc = CMCG_OK;
    unsigned char *buf = NULL;
    long sz = -1;
    if (fseek(fp, 0, SEEK_END) == 0) sz = ftell(fp);
    if (sz <= 0 || fseek(fp, 0, SEEK_SET) != 0) rc = CMCG_ERR_IO;
    if (!rc && !(buf = (unsigned char *)malloc((size_t)sz))) rc = CMCG_ERR_NOMEM;
    if (!rc && fread(buf, 1, (size_t)sz, fp) != (size_t)sz) rc = CMCG_ERR_IO;
    fclose(fp);
    if (rc) {
        free(buf);
        return rc;
    }
    const H5File f = {buf, (size_t)sz};
    H5Dataset od, bd;
    uint64_t ooh = 0, boh = 0;
    rc = open_dataset(&f, "CLUS_OBJ_DATA", "block0_values", &od, &ooh);
    if (!rc) rc = open_dataset(&f, "CLUS_BINARY_DATA", "block0_values", &bd, &boh);
    double nobj = 0, nbin = 0;
    if (!rc) rc = attribute(&f, ooh, "NOBJ", &nobj);
    if (!rc) rc = attribute(&f, ooh, "NBINARY", &nbin);
    if (!rc) rc = attribute(&f, ooh, "MCLUS", &info->mclus);
    if (!rc) rc = attribute(&f, ooh, "RVIR", &info->rvir);
    if (!rc) rc = attribute(&f, ooh, "RTID", &info->rtid);
    if (!rc) rc = attribute(&f, ooh, "Z", &info->z);
    if (!rc) {
        info->nobj = (long)nobj;
        info->nbinary = (long)nbin;
        info->obj_rows = (long)od.dims[0];
        info->obj_cols = (long)od.dims[1];
        info->bin_rows = (long)bd.dims[0];
        info->bin_cols = (long)bd.dims[1];
        /* the reference's loader indexes 8 object and 11 binary columns */
        if (info->obj_cols != 8 || info->bin_cols != 11) rc = CMCG_ERR_FORMAT;
    }
    if (!rc) rc = copy_table(&f, &od, obj, obj_cap_rows);
    if (!rc) rc = copy_table(&f, &bd, bin, bin_cap_rows);
    free(buf);
    return rc;
}
