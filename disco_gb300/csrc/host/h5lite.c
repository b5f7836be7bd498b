/*
 * h5lite.c -- the HDF5 subset of h5lite.h, from the HDF5 File Format
 * Specification 3.0 (superblock II.A, object header IV.A.1.b, messages
 * IV.A.2: dataspace 0x0001, link info 0x0002, datatype 0x0003, fill value
 * 0x0005, link 0x0006, data layout 0x0008, group info 0x000A; global heap
 * III.E) and Bob Jenkins' public-domain lookup3 hash (hashlittle), which
 * HDF5 uses for its metadata checksums.
 */
#define _FILE_OFFSET_BITS 64
#include "h5lite.h"

#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define H5L_UNDEF 0xffffffffffffffffULL
#define H5L_MAXRANK 4

/* ---- lookup3 hashlittle --------------------------------------------------- */
static uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }

uint32_t h5l_lookup3(const void *key, size_t length, uint32_t initval)
{
   const uint8_t *k = (const uint8_t *)key;
   uint32_t a, b, c;
   a = b = c = 0xdeadbeefu + (uint32_t)length + initval;
   while (length > 12) {
      a += (uint32_t)k[0] | (uint32_t)k[1] << 8 | (uint32_t)k[2] << 16 | (uint32_t)k[3] << 24;
      b += (uint32_t)k[4] | (uint32_t)k[5] << 8 | (uint32_t)k[6] << 16 | (uint32_t)k[7] << 24;
      c += (uint32_t)k[8] | (uint32_t)k[9] << 8 | (uint32_t)k[10] << 16 | (uint32_t)k[11] << 24;
      /* mix */
      a -= c; a ^= rotl32(c, 4);  c += b;
      b -= a; b ^= rotl32(a, 6);  a += c;
      c -= b; c ^= rotl32(b, 8);  b += a;
      a -= c; a ^= rotl32(c, 16); c += b;
      b -= a; b ^= rotl32(a, 19); a += c;
      c -= b; c ^= rotl32(b, 4);  b += a;
      length -= 12;
      k += 12;
   }
   if (length == 0) return c;
   /* the last 1..12 bytes, little-endian into a, b, c */
   uint32_t w[3] = {0, 0, 0};
   for (size_t i = 0; i < length; ++i) w[i / 4] |= (uint32_t)k[i] << (8 * (i % 4));
   a += w[0]; b += w[1]; c += w[2];
   /* final */
   c ^= b; c -= rotl32(b, 14);
   a ^= c; a -= rotl32(c, 11);
   b ^= a; b -= rotl32(a, 25);
   c ^= b; c -= rotl32(b, 16);
   a ^= c; a -= rotl32(c, 4);
   b ^= a; b -= rotl32(a, 14);
   c ^= b; c -= rotl32(b, 24);
   return c;
}

/* ---- little-endian byte buffer ------------------------------------------- */
typedef struct { uint8_t *p; size_t n, cap; int err; } buf_t;

static void put(buf_t *b, const void *src, size_t n)
{
   if (b->err) return;
   if (b->n + n > b->cap) {
      size_t cap = b->cap ? b->cap : 256;
      while (cap < b->n + n) cap *= 2;
      uint8_t *q = (uint8_t *)realloc(b->p, cap);
      if (!q) { b->err = 1; return; }
      b->p = q;
      b->cap = cap;
   }
   if (src) memcpy(b->p + b->n, src, n); else memset(b->p + b->n, 0, n);
   b->n += n;
}
static void put_u(buf_t *b, uint64_t v, int nbytes)
{
   uint8_t t[8];
   for (int i = 0; i < nbytes; ++i) t[i] = (uint8_t)(v >> (8 * i));
   put(b, t, (size_t)nbytes);
}
static uint64_t get_u(const uint8_t *p, int nbytes)
{
   uint64_t v = 0;
   for (int i = 0; i < nbytes; ++i) v |= (uint64_t)p[i] << (8 * i);
   return v;
}

/* ---- writer ---------------------------------------------------------------- */
typedef struct { char name[64]; int group; int id; } wlink;   /* id: group id or dataset index */
typedef struct {
   char name[64];
   wlink *links; int nlinks, caplinks;
   uint64_t addr, ohsize;
} wgroup;
typedef struct {
   char name[64];
   int type, rank;
   uint64_t dims[H5L_MAXRANK], n;
   const void *data;
   uint64_t addr, ohsize, data_addr, data_size;
   uint64_t heap_first;           /* VSTR: index of the first heap object */
} wdset;
struct h5w {
   wgroup *g; int ng, capg;
   wdset *d; int nd, capd;
};

static size_t type_msg_size(int type) { return type == H5L_I32 ? 12 : 20; }
static size_t elem_size(int type) { return type == H5L_I32 ? 4 : type == H5L_F64 ? 8 : 16; }

static int add_link(wgroup *g, const char *name, int is_group, int id)
{
   for (int i = 0; i < g->nlinks; ++i)
      if (!strcmp(g->links[i].name, name)) return -EEXIST;
   if (g->nlinks == g->caplinks) {
      int cap = g->caplinks ? 2 * g->caplinks : 16;
      wlink *q = (wlink *)realloc(g->links, (size_t)cap * sizeof(wlink));
      if (!q) return -ENOMEM;
      g->links = q;
      g->caplinks = cap;
   }
   wlink *l = &g->links[g->nlinks++];
   snprintf(l->name, sizeof l->name, "%s", name);
   l->group = is_group;
   l->id = id;
   return 0;
}

h5w *h5w_create(void)
{
   h5w *w = (h5w *)calloc(1, sizeof(h5w));
   if (!w) return NULL;
   w->g = (wgroup *)calloc(8, sizeof(wgroup));
   if (!w->g) { free(w); return NULL; }
   w->capg = 8;
   w->ng = 1;   /* the root group */
   return w;
}

void h5w_abort(h5w *w)
{
   if (!w) return;
   for (int i = 0; i < w->ng; ++i) free(w->g[i].links);
   free(w->g);
   free(w->d);
   free(w);
}

int h5w_group(h5w *w, const char *name)
{
   if (!w || !name) return -EINVAL;
   if (!name[0] || !strcmp(name, "/")) return 0;
   if (strlen(name) >= 64 || strchr(name, '/')) return -EINVAL;
   for (int i = 1; i < w->ng; ++i)
      if (!strcmp(w->g[i].name, name)) return i;
   if (w->ng == w->capg) {
      wgroup *q = (wgroup *)realloc(w->g, (size_t)(2 * w->capg) * sizeof(wgroup));
      if (!q) return -ENOMEM;
      memset(q + w->capg, 0, (size_t)w->capg * sizeof(wgroup));
      w->g = q;
      w->capg *= 2;
   }
   int id = w->ng;
   int rc = add_link(&w->g[0], name, 1, id);
   if (rc) return rc;
   ++w->ng;
   snprintf(w->g[id].name, sizeof w->g[id].name, "%s", name);
   return id;
}

int h5w_dataset(h5w *w, int group, const char *name, int type, int rank,
                const uint64_t *dims, const void *data)
{
   if (!w || !name || group < 0 || group >= w->ng || rank < 0 || rank > H5L_MAXRANK ||
       (rank > 0 && !dims) || (type != H5L_I32 && type != H5L_F64 && type != H5L_VSTR) ||
       !name[0] || strlen(name) >= 64 || strchr(name, '/'))
      return -EINVAL;
   uint64_t n = 1;
   for (int i = 0; i < rank; ++i) n *= dims[i];
   if (n > 0 && !data) return -EINVAL;
   if (w->nd == w->capd) {
      int cap = w->capd ? 2 * w->capd : 64;
      wdset *q = (wdset *)realloc(w->d, (size_t)cap * sizeof(wdset));
      if (!q) return -ENOMEM;
      w->d = q;
      w->capd = cap;
   }
   int rc = add_link(&w->g[group], name, 0, w->nd);
   if (rc) return rc;
   wdset *d = &w->d[w->nd++];
   memset(d, 0, sizeof *d);
   snprintf(d->name, sizeof d->name, "%s", name);
   d->type = type;
   d->rank = rank;
   for (int i = 0; i < rank; ++i) d->dims[i] = dims[i];
   d->n = n;
   d->data = data;
   return 0;
}

/* object header v2: "OHDR", version, flags (chunk-size field of 4 bytes),
 * chunk size, messages (type, size, flags, data), checksum */
static void oh_begin(buf_t *b) { put(b, "OHDR", 4); put_u(b, 2, 1); put_u(b, 2, 1); put_u(b, 0, 4); }
static void oh_msg(buf_t *b, int type, size_t size) { put_u(b, (uint64_t)type, 1); put_u(b, size, 2); put_u(b, 0, 1); }
static void oh_end(buf_t *b, size_t start)
{
   if (b->err) return;
   uint64_t chunk = b->n - start - 10;
   for (int i = 0; i < 4; ++i) b->p[start + 6 + i] = (uint8_t)(chunk >> (8 * i));
   put_u(b, h5l_lookup3(b->p + start, b->n - start, 0), 4);
}

static size_t link_msg_size(const char *name) { return 2 + 1 + strlen(name) + 8; }

static uint64_t group_oh_size(const wgroup *g)
{
   uint64_t s = 10 + 4;                 /* prefix + checksum */
   s += 4 + 18;                         /* link info */
   s += 4 + 6;                          /* group info with phase-change values */
   for (int i = 0; i < g->nlinks; ++i) s += 4 + link_msg_size(g->links[i].name);
   return s;
}
static uint64_t dset_oh_size(const wdset *d)
{
   uint64_t s = 10 + 4;
   s += 4 + 4 + 8 * (uint64_t)d->rank;  /* dataspace v2 */
   s += 4 + type_msg_size(d->type);     /* datatype */
   s += 4 + 4;                          /* fill value v2, undefined */
   s += 4 + 18;                         /* contiguous layout v3 */
   return s;
}

static void write_type(buf_t *b, int type)
{
   if (type == H5L_I32) {               /* fixed-point v1, LE, signed */
      put_u(b, 0x10, 1); put_u(b, 0x08, 1); put_u(b, 0, 2); put_u(b, 4, 4);
      put_u(b, 0, 2); put_u(b, 32, 2);
   } else if (type == H5L_F64) {        /* floating-point v1, LE, implied MSB, sign at bit 63 */
      put_u(b, 0x11, 1); put_u(b, 0x20, 1); put_u(b, 63, 1); put_u(b, 0, 1); put_u(b, 8, 4);
      put_u(b, 0, 2); put_u(b, 64, 2); put_u(b, 52, 1); put_u(b, 11, 1); put_u(b, 0, 1);
      put_u(b, 52, 1); put_u(b, 1023, 4);
   } else {                             /* variable-length v1: string, null-terminated, ASCII */
      put_u(b, 0x19, 1); put_u(b, 0x01, 1); put_u(b, 0, 2); put_u(b, 16, 4);
      /* base type: 1-byte unsigned fixed-point */
      put_u(b, 0x10, 1); put_u(b, 0x00, 1); put_u(b, 0, 2); put_u(b, 1, 4);
      put_u(b, 0, 2); put_u(b, 8, 2);
   }
}

static uint64_t pad8(uint64_t x) { return (x + 7) & ~(uint64_t)7; }

int h5w_close(h5w *w, const char *path)
{
   if (!w || !path) { h5w_abort(w); return -EINVAL; }
   int rc = 0;
   FILE *f = NULL;
   buf_t meta = {0}, heap = {0};
   /* ---- layout: superblock, object headers, global heap, raw data */
   uint64_t at = 48;
   for (int i = 0; i < w->ng; ++i) { w->g[i].addr = at; w->g[i].ohsize = group_oh_size(&w->g[i]); at += w->g[i].ohsize; }
   for (int i = 0; i < w->nd; ++i) { w->d[i].addr = at; w->d[i].ohsize = dset_oh_size(&w->d[i]); at += w->d[i].ohsize; }
   /* global heap collection: one object per string, 16-byte object headers,
    * data padded to 8 bytes, the rest free space (object 0); at least 4 KiB */
   uint64_t heap_addr = H5L_UNDEF, heap_used = 16, nobj = 0;
   for (int i = 0; i < w->nd; ++i) {
      wdset *d = &w->d[i];
      if (d->type != H5L_VSTR) continue;
      d->heap_first = nobj + 1;
      const char *const *s = (const char *const *)d->data;
      for (uint64_t e = 0; e < d->n; ++e) heap_used += 16 + pad8(strlen(s[e] ? s[e] : ""));
      nobj += d->n;
   }
   if (nobj + 1 > 65535) { rc = -E2BIG; goto done; }
   uint64_t heap_size = 0;
   if (nobj) {
      heap_addr = at;
      heap_size = heap_used + 16 > 4096 ? pad8(heap_used + 16) : 4096;
      at += heap_size;
   }
   at = pad8(at);
   for (int i = 0; i < w->nd; ++i) {
      wdset *d = &w->d[i];
      d->data_size = d->n * elem_size(d->type);
      d->data_addr = d->n ? at : H5L_UNDEF;
      at = pad8(at + d->data_size);
   }
   const uint64_t eof = at;

   /* ---- superblock v2 */
   put(&meta, "\x89HDF\r\n\x1a\n", 8);
   put_u(&meta, 2, 1); put_u(&meta, 8, 1); put_u(&meta, 8, 1); put_u(&meta, 0, 1);
   put_u(&meta, 0, 8);                 /* base address */
   put_u(&meta, H5L_UNDEF, 8);         /* no superblock extension */
   put_u(&meta, eof, 8);
   put_u(&meta, w->g[0].addr, 8);
   if (!meta.err) put_u(&meta, h5l_lookup3(meta.p, meta.n, 0), 4);
   /* ---- groups */
   for (int i = 0; i < w->ng; ++i) {
      const wgroup *g = &w->g[i];
      size_t s0 = meta.n;
      oh_begin(&meta);
      oh_msg(&meta, 0x0002, 18);       /* link info: no creation order, compact */
      put_u(&meta, 0, 1); put_u(&meta, 0, 1); put_u(&meta, H5L_UNDEF, 8); put_u(&meta, H5L_UNDEF, 8);
      oh_msg(&meta, 0x000A, 6);        /* group info: phase-change values */
      int maxc = g->nlinks > 8 ? g->nlinks : 8;
      put_u(&meta, 0, 1); put_u(&meta, 1, 1); put_u(&meta, (uint64_t)maxc, 2); put_u(&meta, 6, 2);
      for (int l = 0; l < g->nlinks; ++l) {
         const wlink *lk = &g->links[l];
         size_t len = strlen(lk->name);
         oh_msg(&meta, 0x0006, link_msg_size(lk->name));
         put_u(&meta, 1, 1); put_u(&meta, 0, 1);   /* version 1; hard link, 1-byte name length */
         put_u(&meta, len, 1);
         put(&meta, lk->name, len);
         put_u(&meta, lk->group ? w->g[lk->id].addr : w->d[lk->id].addr, 8);
      }
      oh_end(&meta, s0);
      if (!meta.err && meta.n - s0 != g->ohsize) { rc = -EFAULT; goto done; }
   }
   /* ---- datasets */
   for (int i = 0; i < w->nd; ++i) {
      const wdset *d = &w->d[i];
      size_t s0 = meta.n;
      oh_begin(&meta);
      oh_msg(&meta, 0x0001, 4 + 8 * (size_t)d->rank);
      put_u(&meta, 2, 1); put_u(&meta, (uint64_t)d->rank, 1); put_u(&meta, 0, 1);
      put_u(&meta, d->rank ? 1 : 0, 1);
      for (int r = 0; r < d->rank; ++r) put_u(&meta, d->dims[r], 8);
      oh_msg(&meta, 0x0003, type_msg_size(d->type));
      write_type(&meta, d->type);
      oh_msg(&meta, 0x0005, 4);        /* fill value v2: late allocation, write if set, undefined */
      put_u(&meta, 2, 1); put_u(&meta, 2, 1); put_u(&meta, 2, 1); put_u(&meta, 0, 1);
      oh_msg(&meta, 0x0008, 18);       /* layout v3, contiguous */
      put_u(&meta, 3, 1); put_u(&meta, 1, 1); put_u(&meta, d->data_addr, 8); put_u(&meta, d->data_size, 8);
      oh_end(&meta, s0);
      if (!meta.err && meta.n - s0 != d->ohsize) { rc = -EFAULT; goto done; }
   }
   /* ---- global heap */
   if (nobj) {
      put(&heap, "GCOL", 4); put_u(&heap, 1, 1); put_u(&heap, 0, 3); put_u(&heap, heap_size, 8);
      uint64_t idx = 1;
      for (int i = 0; i < w->nd; ++i) {
         const wdset *d = &w->d[i];
         if (d->type != H5L_VSTR) continue;
         const char *const *s = (const char *const *)d->data;
         for (uint64_t e = 0; e < d->n; ++e, ++idx) {
            const char *str = s[e] ? s[e] : "";
            size_t len = strlen(str);
            put_u(&heap, idx, 2); put_u(&heap, 0, 2); put_u(&heap, 0, 4); put_u(&heap, len, 8);
            put(&heap, str, len);
            put(&heap, NULL, (size_t)(pad8(len) - len));
         }
      }
      uint64_t rest = heap_size - heap.n;   /* >= 16 by construction */
      put_u(&heap, 0, 2); put_u(&heap, 0, 2); put_u(&heap, 0, 4); put_u(&heap, rest, 8);
      put(&heap, NULL, (size_t)(rest - 16));
   }
   if (meta.err || heap.err) { rc = -ENOMEM; goto done; }
   if (meta.n + heap.n != (nobj ? heap_addr + heap_size : meta.n)) { rc = -EFAULT; goto done; }

   f = fopen(path, "wb");
   if (!f) { rc = -errno; goto done; }
   if (fwrite(meta.p, 1, meta.n, f) != meta.n) { rc = -EIO; goto done; }
   if (heap.n && fwrite(heap.p, 1, heap.n, f) != heap.n) { rc = -EIO; goto done; }
   uint64_t pos = meta.n + heap.n;
   static const uint8_t zeros[8] = {0};
   for (int i = 0; i < w->nd; ++i) {
      const wdset *d = &w->d[i];
      if (!d->n) continue;
      if (d->data_addr > pos && fwrite(zeros, 1, (size_t)(d->data_addr - pos), f) != d->data_addr - pos) { rc = -EIO; goto done; }
      pos = d->data_addr;
      if (d->type == H5L_VSTR) {
         const char *const *s = (const char *const *)d->data;
         for (uint64_t e = 0; e < d->n; ++e) {
            buf_t el = {0};
            put_u(&el, strlen(s[e] ? s[e] : ""), 4);
            put_u(&el, heap_addr, 8);
            put_u(&el, d->heap_first + e, 4);
            int bad = el.err || fwrite(el.p, 1, 16, f) != 16;
            free(el.p);
            if (bad) { rc = -EIO; goto done; }
         }
      } else if (fwrite(d->data, elem_size(d->type), (size_t)d->n, f) != d->n) {
         rc = -EIO;
         goto done;
      }
      pos += d->data_size;
   }
   if (eof > pos && fwrite(zeros, 1, (size_t)(eof - pos), f) != eof - pos) { rc = -EIO; goto done; }
done:
   if (f && fclose(f) != 0 && rc == 0) rc = -EIO;
   free(meta.p);
   free(heap.p);
   h5w_abort(w);
   return rc;
}

/* ---- reader ---------------------------------------------------------------- */
struct h5r {
   FILE *f;
   uint64_t eof, root;
};

static int rd(h5r *r, uint64_t addr, void *dst, size_t n)
{
   if (addr > r->eof || n > r->eof - addr) return -1;
   if (fseeko(r->f, (off_t)addr, SEEK_SET) != 0) return -1;
   return fread(dst, 1, n, r->f) == n ? 0 : -1;
}

void h5r_close(h5r *r)
{
   if (!r) return;
   if (r->f) fclose(r->f);
   free(r);
}

h5r *h5r_open(const char *path, char *err, size_t nerr)
{
   h5r *r = (h5r *)calloc(1, sizeof(h5r));
   uint8_t sb[48];
   const char *why = NULL;
   if (!r) { why = "out of memory"; goto fail; }
   r->f = fopen(path, "rb");
   if (!r->f) { why = "cannot open file"; goto fail; }
   if (fseeko(r->f, 0, SEEK_END) != 0) { why = "cannot seek"; goto fail; }
   r->eof = (uint64_t)ftello(r->f);
   if (rd(r, 0, sb, 9) != 0 || memcmp(sb, "\x89HDF\r\n\x1a\n", 8) != 0) { why = "not an HDF5 file"; goto fail; }
   if (sb[8] != 2 && sb[8] != 3) { why = "unsupported superblock version (2 or 3 only)"; goto fail; }
   if (rd(r, 0, sb, 48) != 0) { why = "truncated superblock"; goto fail; }
   if (sb[9] != 8 || sb[10] != 8) { why = "unsupported offset/length size"; goto fail; }
   if (h5l_lookup3(sb, 44, 0) != (uint32_t)get_u(sb + 44, 4)) { why = "superblock checksum mismatch"; goto fail; }
   if (get_u(sb + 12, 8) != 0) { why = "non-zero base address"; goto fail; }
   if (get_u(sb + 28, 8) > r->eof) { why = "file shorter than its end-of-file address"; goto fail; }
   r->root = get_u(sb + 36, 8);
   return r;
fail:
   if (err && nerr) snprintf(err, nerr, "%s: %s", path, why);
   h5r_close(r);
   return NULL;
}

/* One object header v2 in a malloc'd buffer (checksum verified): messages
 * from offset m0 to n, each with a 2-byte creation order if corder. */
typedef struct { uint8_t *p; size_t n, m0; int corder; } ohbuf;

static int read_oh(h5r *r, uint64_t addr, ohbuf *oh)
{
   uint8_t pre[6 + 16 + 4 + 8];
   if (rd(r, addr, pre, 6) != 0 || memcmp(pre, "OHDR", 4) != 0 || pre[4] != 2) return -1;
   int flags = pre[5];
   size_t hdr = 6 + ((flags & 0x20) ? 16 : 0) + ((flags & 0x10) ? 4 : 0);
   int csz = 1 << (flags & 3);
   if (rd(r, addr, pre, hdr + (size_t)csz) != 0) return -1;
   uint64_t chunk = get_u(pre + hdr, csz);
   size_t total = hdr + (size_t)csz + (size_t)chunk + 4;
   if (chunk > r->eof) return -1;
   uint8_t *p = (uint8_t *)malloc(total);
   if (!p) return -1;
   if (rd(r, addr, p, total) != 0 || h5l_lookup3(p, total - 4, 0) != (uint32_t)get_u(p + total - 4, 4)) {
      free(p);
      return -1;
   }
   oh->p = p;
   oh->n = total - 4;
   oh->m0 = hdr + (size_t)csz;
   oh->corder = (flags & 0x04) != 0;
   return 0;
}

/* Iterates the messages of an object header: calls fn(type, data, size). */
typedef int (*msg_fn)(int type, const uint8_t *d, size_t n, void *ctx);
static int each_msg(const ohbuf *oh, msg_fn fn, void *ctx)
{
   size_t at = oh->m0;
   const size_t hsz = 4 + (oh->corder ? 2 : 0);
   while (at + hsz <= oh->n) {
      int type = oh->p[at];
      size_t sz = (size_t)get_u(oh->p + at + 1, 2);
      if (at + hsz + sz > oh->n) return -1;
      if (type == 0x0010) return -2;   /* continuation: not in this subset */
      int rc = fn(type, oh->p + at + hsz, sz, ctx);
      if (rc) return rc;
      at += hsz + sz;
   }
   return 0;
}

typedef struct { const char *name; size_t len; uint64_t addr; int found; } link_ctx;
static int link_cb(int type, const uint8_t *d, size_t n, void *vctx)
{
   link_ctx *c = (link_ctx *)vctx;
   if (type != 0x0006 || n < 2 || d[0] != 1) return 0;
   int fl = d[1];
   size_t at = 2;
   int ltype = 0;
   if (fl & 0x08) ltype = d[at++];
   if (fl & 0x04) at += 8;
   if (fl & 0x10) at += 1;
   int lsz = 1 << (fl & 3);
   if (at + (size_t)lsz > n) return -1;
   size_t len = (size_t)get_u(d + at, lsz);
   at += (size_t)lsz;
   if (at + len > n) return -1;
   if (ltype == 0 && len == c->len && !memcmp(d + at, c->name, len) && at + len + 8 <= n) {
      c->addr = get_u(d + at + len, 8);
      c->found = 1;
   }
   return 0;
}

/* Address of the object at "a/b/c" below the root. */
static int resolve(h5r *r, const char *path, uint64_t *addr)
{
   uint64_t cur = r->root;
   const char *s = path;
   while (*s == '/') ++s;
   while (*s) {
      const char *e = strchr(s, '/');
      size_t len = e ? (size_t)(e - s) : strlen(s);
      ohbuf oh;
      if (read_oh(r, cur, &oh) != 0) return -1;
      link_ctx c = {s, len, 0, 0};
      int rc = each_msg(&oh, link_cb, &c);
      free(oh.p);
      if (rc || !c.found) return -1;
      cur = c.addr;
      s += len;
      while (*s == '/') ++s;
   }
   *addr = cur;
   return 0;
}

typedef struct {
   int rank, have_space, have_type, have_layout;
   uint64_t dims[H5L_MAXRANK];
   int cls, size, is_signed, vstr;
   int layout;                /* 0 compact, 1 contiguous */
   uint64_t daddr, dsize;
   const uint8_t *compact;    /* into the header buffer */
} dsinfo;

static int ds_cb(int type, const uint8_t *d, size_t n, void *vctx)
{
   dsinfo *x = (dsinfo *)vctx;
   if (type == 0x0001) {                 /* dataspace v1 or v2 */
      if (n < 4) return -1;
      int ver = d[0], rank = d[1], fl = d[2];
      size_t at = ver == 1 ? 8 : 4;
      if ((ver != 1 && ver != 2) || rank > H5L_MAXRANK || at + 8 * (size_t)rank > n) return -1;
      if (ver == 2 && d[3] == 2) return -1;   /* null dataspace */
      (void)fl;
      x->rank = rank;
      for (int i = 0; i < rank; ++i) x->dims[i] = get_u(d + at + 8 * (size_t)i, 8);
      x->have_space = 1;
   } else if (type == 0x0003) {          /* datatype */
      if (n < 8) return -1;
      x->cls = d[0] & 0x0f;
      x->size = (int)get_u(d + 4, 4);
      if (x->cls == 0) {
         if (d[1] & 0x01) return -1;     /* big-endian */
         x->is_signed = (d[1] >> 3) & 1;
      } else if (x->cls == 1) {
         if ((d[1] & 0x01) || (d[1] & 0x40) || x->size != 8) return -1;
      } else if (x->cls == 9) {
         if ((d[1] & 0x0f) != 1) return -1;   /* sequences: not in this subset */
         x->vstr = 1;
      } else {
         return -1;
      }
      x->have_type = 1;
   } else if (type == 0x0008) {          /* layout v3 */
      if (n < 2 || d[0] != 3) return -1;
      if (d[1] == 1 && n >= 18) {
         x->layout = 1;
         x->daddr = get_u(d + 2, 8);
         x->dsize = get_u(d + 10, 8);
      } else if (d[1] == 0 && n >= 4) {
         x->layout = 0;
         x->dsize = get_u(d + 2, 2);
         if (4 + x->dsize > n) return -1;
         x->compact = d + 4;
      } else {
         return -1;                      /* chunked / virtual */
      }
      x->have_layout = 1;
   }
   return 0;
}

static int ds_open(h5r *r, const char *path, dsinfo *x, ohbuf *oh)
{
   uint64_t addr;
   memset(x, 0, sizeof *x);
   if (resolve(r, path, &addr) != 0 || read_oh(r, addr, oh) != 0) return -1;
   if (each_msg(oh, ds_cb, x) != 0 || !x->have_space || !x->have_type || !x->have_layout) {
      free(oh->p);
      return -1;
   }
   return 0;
}

int h5r_dims(h5r *r, const char *path, uint64_t *dims, int maxrank, int *type)
{
   dsinfo x;
   ohbuf oh;
   if (!r || !path || ds_open(r, path, &x, &oh) != 0) return -1;
   free(oh.p);
   for (int i = 0; i < x.rank && i < maxrank; ++i) dims[i] = x.dims[i];
   if (type) *type = x.vstr ? H5L_VSTR : x.cls == 1 ? H5L_F64 : H5L_I32;
   return x.rank;
}

long h5r_read(h5r *r, const char *path, int type, long row0, long nrow, void *out)
{
   dsinfo x;
   ohbuf oh;
   if (!r || !path || !out || (type != H5L_I32 && type != H5L_F64)) return -1;
   if (ds_open(r, path, &x, &oh) != 0) return -1;
   long rc = -1;
   uint64_t rows = x.rank ? x.dims[0] : 1, rowlen = 1;
   for (int i = 1; i < x.rank; ++i) rowlen *= x.dims[i];
   if (nrow < 0) { row0 = 0; nrow = (long)rows; }
   const int es = x.size;
   if (x.vstr || row0 < 0 || (uint64_t)row0 + (uint64_t)nrow > rows ||
       (x.cls == 0 && es != 1 && es != 2 && es != 4 && es != 8)) goto done;
   {
      const uint64_t nel = (uint64_t)nrow * rowlen, off = (uint64_t)row0 * rowlen * (uint64_t)es;
      if (off + nel * (uint64_t)es > x.dsize) goto done;
      uint8_t *raw = (uint8_t *)malloc(nel * (uint64_t)es + 1);
      if (!raw) goto done;
      int ok;
      if (x.layout == 1) ok = x.daddr == H5L_UNDEF ? (memset(raw, 0, nel * (uint64_t)es), 1)
                                                    : rd(r, x.daddr + off, raw, nel * (uint64_t)es) == 0;
      else ok = (memcpy(raw, x.compact + off, nel * (uint64_t)es), 1);
      if (ok) {
         for (uint64_t i = 0; i < nel; ++i) {
            const uint8_t *p = raw + i * (uint64_t)es;
            double v;
            if (x.cls == 1) {
               uint64_t bits = get_u(p, 8);
               memcpy(&v, &bits, 8);
            } else {
               uint64_t u = get_u(p, es);
               if (x.is_signed && es < 8 && (u >> (8 * es - 1)) & 1) u |= ~(uint64_t)0 << (8 * es);
               v = x.is_signed ? (double)(int64_t)u : (double)u;
            }
            if (type == H5L_F64) ((double *)out)[i] = v;
            else ((int *)out)[i] = (int)v;
         }
         rc = (long)nel;
      }
      free(raw);
   }
done:
   free(oh.p);
   return rc;
}

int h5r_read_str(h5r *r, const char *path, char *buf, size_t n)
{
   dsinfo x;
   ohbuf oh;
   if (!r || !path || !buf || !n) return -1;
   if (ds_open(r, path, &x, &oh) != 0) return -1;
   int rc = -1;
   uint8_t el[16], hh[16];
   if (!x.vstr || x.size != 16 || x.dsize < 16) goto done;
   if (x.layout == 1 ? rd(r, x.daddr, el, 16) != 0 : (memcpy(el, x.compact, 16), 0)) goto done;
   {
      const uint64_t len = get_u(el, 4), gaddr = get_u(el + 4, 8), idx = get_u(el + 12, 4);
      if (len == 0) { buf[0] = 0; rc = 0; goto done; }
      if (rd(r, gaddr, hh, 16) != 0 || memcmp(hh, "GCOL", 4) != 0 || hh[4] != 1) goto done;
      const uint64_t csize = get_u(hh + 8, 8);
      uint64_t at = 16;
      while (at + 16 <= csize) {
         uint8_t oh16[16];
         if (rd(r, gaddr + at, oh16, 16) != 0) goto done;
         const uint64_t oi = get_u(oh16, 2), os = get_u(oh16 + 8, 8);
         if (oi == 0) break;
         if (oi == idx) {
            if (os < len || len >= n) goto done;
            if (rd(r, gaddr + at + 16, buf, (size_t)len) != 0) goto done;
            buf[len] = 0;
            rc = 0;
            goto done;
         }
         at += 16 + pad8(os);
      }
   }
done:
   free(oh.p);
   return rc;
}
