/*
 * h5lite.h -- a minimal HDF5 file writer and reader for the checkpoint
 * layout of the reference's Output/h5out.c and Restart/h5in.c.
 *
 * Neither machine this library targets has the HDF5 library, so the subset
 * the checkpoint needs is written directly from the published HDF5 File
 * Format Specification (version 3.0):
 *   - superblock version 2 (8-byte offsets and lengths, Jenkins lookup3
 *     checksum);
 *   - version 2 object headers, one chunk, with checksum;
 *   - groups with compact link storage (Link Info, Group Info and Link
 *     messages: hard links only);
 *   - datasets with a version 2 dataspace (simple, fixed size), a version 2
 *     fill value message (undefined fill) and a version 3 contiguous layout;
 *   - datatypes: little-endian 32-bit signed integers, IEEE little-endian
 *     doubles, and variable-length ASCII strings, whose characters live in
 *     one global heap collection.
 * The reader accepts files in this subset (the files h5w_close writes); it
 * reports anything else (superblock versions 0/1, old-style symbol-table
 * groups, chunked or compressed data) as unsupported.
 */
#ifndef DISCO_H5LITE_H
#define DISCO_H5LITE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum h5l_type { H5L_I32 = 1, H5L_F64 = 2, H5L_VSTR = 3 };

/* Jenkins lookup3 hashlittle (the HDF5 metadata checksum with initval 0). */
uint32_t h5l_lookup3(const void *key, size_t length, uint32_t initval);

/* ---- writer: declare the tree, then h5w_close lays it out and writes it */
typedef struct h5w h5w;
h5w *h5w_create(void);
/* A group under the root ("Grid").  Returns its id (> 0), or 0 for the
 * root itself when name is "/" or empty; negative on error. */
int h5w_group(h5w *w, const char *name);
/* A dataset in group `group` (an id from h5w_group, 0 = root).  For
 * H5L_I32 / H5L_F64 `data` holds prod(dims) elements in C order; for
 * H5L_VSTR it holds prod(dims) `const char *` (NUL-terminated).  The data
 * must stay valid until h5w_close.  rank is 0..4. */
int h5w_dataset(h5w *w, int group, const char *name, int type, int rank,
                const uint64_t *dims, const void *data);
/* Writes the file and frees the writer.  0 or a negative errno-like code. */
int h5w_close(h5w *w, const char *path);
void h5w_abort(h5w *w);

/* ---- reader */
typedef struct h5r h5r;
h5r *h5r_open(const char *path, char *err, size_t nerr);
void h5r_close(h5r *r);
/* Shape of "group/name" ("Grid/Index"; a root dataset is "name").  Returns
 * the rank (>= 0) and fills dims, or -1 if absent / unsupported. */
int h5r_dims(h5r *r, const char *path, uint64_t *dims, int maxrank, int *type);
/* Reads rows [row0, row0 + nrow) of the dataset (all of it for a rank-0 or
 * rank-1 dataset when nrow < 0) into out as `type` (H5L_I32 or H5L_F64,
 * converted from the file type).  Returns the number of elements read or a
 * negative code. */
long h5r_read(h5r *r, const char *path, int type, long row0, long nrow, void *out);
/* A scalar or 1-element variable-length string dataset, copied into buf. */
int h5r_read_str(h5r *r, const char *path, char *buf, size_t n);

#ifdef __cplusplus
}
#endif
#endif
