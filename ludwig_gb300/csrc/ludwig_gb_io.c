/*****************************************************************************
 *
 *  ludwig_gb_io.c
 *
 *  Snapshot (restart) files in the reference's on-disk format, for one
 *  rank writing one file per object:
 *
 *    lb_io_write / lb_io_read        src/lb_data.c:1716-1830 with the
 *                                    records of lb_write_buf(_ascii),
 *                                    src/lb_data.c:1533-1640
 *    field_io_write / field_io_read  src/field.c:1633-1737 with
 *                                    field_write_buf(_ascii),
 *                                    src/field.c:896-996
 *    hydro_io_write / hydro_io_read  src/hydro.c:941-967 (fields "rho"
 *                                    and "vel")
 *    file names                      io_subfile_name, src/io_subfile.c:186
 *                                    and io_metadata_write,
 *                                    src/io_metadata.c:244-282
 *
 *  The data file holds the sites in x, y, z order (z fastest, the order of
 *  cs_limits_ic/jc/kc in the aggregators), one fixed-length record per
 *  site.  The metadata file is the JSON of io_metadata_to_json
 *  (src/io_metadata.c:159) in the layout cJSON prints it.
 *
 *  The device data are copied through host memory in the reference's
 *  layout (lb_f_to_host etc.), so reduced-precision objects are written as
 *  the doubles of the reference's values.
 *
 *****************************************************************************/

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ludwig_gb.h"
#include "lgb_internal.h"

#define NVEL 19
#define ASCII_NBYTE 23                  /* " %22.15e" */

static int io_fail(const char * what, const char * file) {
  char msg[512];
  snprintf(msg, sizeof(msg), "%s: %s", what, file);
  return lgb_internal_err(LUDWIG_GB_EIO, msg);
}

static int fmt_valid(int f) {
  return f == IO_RECORD_ASCII || f == IO_RECORD_BINARY;
}

/* Record length of one site: nrow rows of ncol values */
static size_t record_bytes(int fmt, int nrow, int ncol) {
  if (fmt == IO_RECORD_BINARY) return (size_t) nrow*ncol*sizeof(double);
  return (size_t) nrow*(ncol*ASCII_NBYTE + 1);
}

static void data_name(char * buf, size_t n, const char * stub, int step) {
  snprintf(buf, n, "%s-%9.9d.%3.3d-%3.3d", stub, step, 1, 1);
}

/* The metadata JSON as cJSON prints it (tabs, no final newline) */
static int write_metadata(const char * stub, const int ntotal[3], int fmt,
			  int count) {
  char file[256];
  snprintf(file, sizeof(file), "%s-metadata.%3.3d-%3.3d", stub, 1, 1);
  FILE * fp = fopen(file, "w");
  if (fp == NULL) return io_fail("cannot open", file);
  const int bin = (fmt == IO_RECORD_BINARY);
  int nw = fprintf(fp,
    "{\n"
    "\t\"coords\":\t{\n"
    "\t\t\"options\":\t{\n"
    "\t\t\t\"System size (total)\":\t[%d, %d, %d],\n"
    "\t\t\t\"Periodic boundaries\":\t[1, 1, 1],\n"
    "\t\t\t\"Left-end limit Lmin\":\t[0.5, 0.5, 0.5]\n"
    "\t\t},\n"
    "\t\t\"lees_edwards\":\t{\n"
    "\t\t\t\"Number of planes\":\t0\n"
    "\t\t}\n"
    "\t},\n"
    "\t\"io_options\":\t{\n"
    "\t\t\"Mode\":\t\"mpiio\",\n"
    "\t\t\"Record format\":\t\"%s\",\n"
    "\t\t\"Metadata version\":\t3,\n"
    "\t\t\"Report\":\tfalse,\n"
    "\t\t\"Asynchronous\":\tfalse,\n"
    "\t\t\"Compression level\":\t0,\n"
    "\t\t\"I/O grid\":\t[1, 1, 1]\n"
    "\t},\n"
    "\t\"io_element\":\t{\n"
    "\t\t\"MPI_Datatype\":\t\"%s\",\n"
    "\t\t\"Size (bytes)\":\t%d,\n"
    "\t\t\"Count\":\t%d,\n"
    "\t\t\"Endianness\":\t\"LITTLE_ENDIAN\"\n"
    "\t},\n"
    "\t\"io_subfile\":\t{\n"
    "\t\t\"Number of files\":\t1,\n"
    "\t\t\"File index\":\t0,\n"
    "\t\t\"Topology\":\t[1, 1, 1],\n"
    "\t\t\"Coordinate\":\t[0, 0, 0],\n"
    "\t\t\"Data ndims\":\t3,\n"
    "\t\t\"File size (sites)\":\t[%d, %d, %d],\n"
    "\t\t\"File offset (sites)\":\t[0, 0, 0]\n"
    "\t}\n"
    "}",
    ntotal[0], ntotal[1], ntotal[2], bin ? "binary" : "ascii",
    bin ? "MPI_DOUBLE" : "MPI_CHAR", bin ? 8 : 1, count,
    ntotal[0], ntotal[1], ntotal[2]);
  if (fclose(fp) != 0 || nw < 0) return io_fail("cannot write", file);
  return LUDWIG_GB_OK;
}

/* Site-major records from a component-major host array a[c][site]:
 * row r of the record holds values c = col*nrow + r, col = 0..ncol-1
 * (lb: rows are velocities, columns distributions; field: one row) */
static int write_data(const char * file, const double * a, long long nsites,
		      int nrow, int ncol, int fmt) {
  FILE * fp = fopen(file, "wb");
  if (fp == NULL) return io_fail("cannot open", file);
  const size_t rec = record_bytes(fmt, nrow, ncol);
  const long long chunk = 4096;
  char * buf = (char *) malloc(rec*chunk + 64);
  if (buf == NULL) { fclose(fp); return io_fail("out of memory for", file); }
  int rc = LUDWIG_GB_OK;
  for (long long i0 = 0; i0 < nsites && rc == LUDWIG_GB_OK; i0 += chunk) {
    const long long n = (nsites - i0 < chunk) ? nsites - i0 : chunk;
    for (long long k = 0; k < n; k++) {
      char * r = buf + k*rec;
      const long long i = i0 + k;
      if (fmt == IO_RECORD_BINARY) {
	double * v = (double *) r;
	for (int col = 0; col < ncol; col++) {
	  for (int row = 0; row < nrow; row++) {
	    v[col*nrow + row] = a[(size_t) (col*nrow + row)*nsites + i];
	  }
	}
      }
      else {
	char * c = r;
	for (int row = 0; row < nrow; row++) {
	  for (int col = 0; col < ncol; col++) {
	    char tmp[64];
	    int np = snprintf(tmp, sizeof(tmp), " %22.15e",
			      a[(size_t) (col*nrow + row)*nsites + i]);
	    if (np != ASCII_NBYTE) rc = io_fail("ascii record overflow", file);
	    memcpy(c, tmp, ASCII_NBYTE);
	    c += ASCII_NBYTE;
	  }
	  *c++ = '\n';
	}
      }
    }
    if (rc == LUDWIG_GB_OK && fwrite(buf, rec, (size_t) n, fp) != (size_t) n) {
      rc = io_fail("short write", file);
    }
  }
  free(buf);
  if (fclose(fp) != 0 && rc == LUDWIG_GB_OK) rc = io_fail("cannot close", file);
  return rc;
}

static int read_data(const char * file, double * a, long long nsites,
		     int nrow, int ncol, int fmt) {
  FILE * fp = fopen(file, "rb");
  if (fp == NULL) return io_fail("cannot open", file);
  const size_t rec = record_bytes(fmt, nrow, ncol);
  const long long chunk = 4096;
  char * buf = (char *) malloc(rec*chunk + 64);
  if (buf == NULL) { fclose(fp); return io_fail("out of memory for", file); }
  int rc = LUDWIG_GB_OK;
  for (long long i0 = 0; i0 < nsites && rc == LUDWIG_GB_OK; i0 += chunk) {
    const long long n = (nsites - i0 < chunk) ? nsites - i0 : chunk;
    if (fread(buf, rec, (size_t) n, fp) != (size_t) n) {
      rc = io_fail("short read (size or format mismatch)", file);
      break;
    }
    for (long long k = 0; k < n && rc == LUDWIG_GB_OK; k++) {
      const char * r = buf + k*rec;
      const long long i = i0 + k;
      if (fmt == IO_RECORD_BINARY) {
	const double * v = (const double *) r;
	for (int c = 0; c < nrow*ncol; c++) a[(size_t) c*nsites + i] = v[c];
      }
      else {
	const char * c = r;
	for (int row = 0; row < nrow; row++) {
	  for (int col = 0; col < ncol; col++) {
	    char tmp[ASCII_NBYTE + 1];
	    memcpy(tmp, c, ASCII_NBYTE);
	    tmp[ASCII_NBYTE] = '\0';
	    if (sscanf(tmp, "%le", a + (size_t) (col*nrow + row)*nsites + i)
		!= 1) {
	      rc = io_fail("bad ascii record", file);
	    }
	    c += ASCII_NBYTE;
	  }
	  c += 1;                                          /* newline */
	}
      }
    }
  }
  if (rc == LUDWIG_GB_OK && fgetc(fp) != EOF) {
    rc = io_fail("file longer than the lattice", file);
  }
  free(buf);
  fclose(fp);
  return rc;
}

int lb_io_record_format_set(lb_t * lb, int iorformat_in, int iorformat_out) {
  int nt[3], ndist;
  lgb_io_state_t * io = NULL;
  int rc = lgb_internal_lb_io(lb, nt, &ndist, &io);
  if (rc) return rc;
  if (!fmt_valid(iorformat_in) || !fmt_valid(iorformat_out)) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "io record format");
  }
  io->fmt_in = iorformat_in;
  io->fmt_out = iorformat_out;
  return LUDWIG_GB_OK;
}

int field_io_record_format_set(field_t * field, int iorformat_in,
			       int iorformat_out) {
  int nt[3], nf;
  const char * name = NULL;
  lgb_io_state_t * io = NULL;
  int rc = lgb_internal_field_io(field, nt, &nf, &name, &io);
  if (rc) return rc;
  if (!fmt_valid(iorformat_in) || !fmt_valid(iorformat_out)) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "io record format");
  }
  io->fmt_in = iorformat_in;
  io->fmt_out = iorformat_out;
  return LUDWIG_GB_OK;
}

/* lb: host array [ndist*19][nsites], distribution d at rows d*19.. */
static int lb_host(lb_t * lb, int ndist, long long n, double ** pa) {
  double * a = (double *) malloc((size_t) ndist*NVEL*n*sizeof(double));
  if (a == NULL) return lgb_internal_err(LUDWIG_GB_ENOMEM, "lb io buffer");
  *pa = a;
  return LUDWIG_GB_OK;
}

int lb_io_write(lb_t * lb, int timestep, io_event_t * event) {
  (void) event;
  int nt[3], ndist;
  lgb_io_state_t * io = NULL;
  int rc = lgb_internal_lb_io(lb, nt, &ndist, &io);
  if (rc) return rc;
  if (timestep < 0 || timestep >= 1000000000) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "lb_io_write: timestep");
  }
  const long long n = (long long) nt[0]*nt[1]*nt[2];
  double * a = NULL;
  if ((rc = lb_host(lb, ndist, n, &a))) return rc;
  rc = lb_f_to_host(lb, a);
  if (rc == 0 && ndist == 2) rc = lb_g_to_host(lb, a + (size_t) NVEL*n);
  if (rc == 0 && !io->meta_written) {
    rc = write_metadata("dist", nt, io->fmt_out, (io->fmt_out ==
	 IO_RECORD_BINARY) ? ndist*NVEL : NVEL*(ndist*ASCII_NBYTE + 1));
    if (rc == 0) io->meta_written = 1;
  }
  if (rc == 0) {
    char file[256];
    data_name(file, sizeof(file), "dist", timestep);
    rc = write_data(file, a, n, NVEL, ndist, io->fmt_out);
  }
  free(a);
  return rc;
}

int lb_io_read(lb_t * lb, int timestep, io_event_t * event) {
  (void) event;
  int nt[3], ndist;
  lgb_io_state_t * io = NULL;
  int rc = lgb_internal_lb_io(lb, nt, &ndist, &io);
  if (rc) return rc;
  if (timestep < 0 || timestep >= 1000000000) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "lb_io_read: timestep");
  }
  const long long n = (long long) nt[0]*nt[1]*nt[2];
  double * a = NULL;
  if ((rc = lb_host(lb, ndist, n, &a))) return rc;
  char file[256];
  data_name(file, sizeof(file), "dist", timestep);
  rc = read_data(file, a, n, NVEL, ndist, io->fmt_in);
  if (rc == 0) rc = lb_f_from_host(lb, a);
  if (rc == 0 && ndist == 2) rc = lb_g_from_host(lb, a + (size_t) NVEL*n);
  free(a);
  return rc;
}

int field_io_write(field_t * field, int timestep, io_event_t * event) {
  (void) event;
  int nt[3], nf;
  const char * name = NULL;
  lgb_io_state_t * io = NULL;
  int rc = lgb_internal_field_io(field, nt, &nf, &name, &io);
  if (rc) return rc;
  if (timestep < 0 || timestep >= 1000000000) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "field_io_write: timestep");
  }
  const long long n = (long long) nt[0]*nt[1]*nt[2];
  double * a = (double *) malloc((size_t) nf*n*sizeof(double));
  if (a == NULL) return lgb_internal_err(LUDWIG_GB_ENOMEM, "field io buffer");
  rc = field_to_host(field, a);
  if (rc == 0 && !io->meta_written) {
    rc = write_metadata(name, nt, io->fmt_out, (io->fmt_out ==
	 IO_RECORD_BINARY) ? nf : nf*ASCII_NBYTE + 1);
    if (rc == 0) io->meta_written = 1;
  }
  if (rc == 0) {
    char file[256];
    data_name(file, sizeof(file), name, timestep);
    rc = write_data(file, a, n, 1, nf, io->fmt_out);
  }
  free(a);
  return rc;
}

int field_io_read(field_t * field, int timestep, io_event_t * event) {
  (void) event;
  int nt[3], nf;
  const char * name = NULL;
  lgb_io_state_t * io = NULL;
  int rc = lgb_internal_field_io(field, nt, &nf, &name, &io);
  if (rc) return rc;
  if (timestep < 0 || timestep >= 1000000000) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "field_io_read: timestep");
  }
  const long long n = (long long) nt[0]*nt[1]*nt[2];
  double * a = (double *) malloc((size_t) nf*n*sizeof(double));
  if (a == NULL) return lgb_internal_err(LUDWIG_GB_ENOMEM, "field io buffer");
  char file[256];
  data_name(file, sizeof(file), name, timestep);
  rc = read_data(file, a, n, 1, nf, io->fmt_in);
  if (rc == 0) rc = field_from_host(field, a);
  free(a);
  return rc;
}

int hydro_io_record_format_set(hydro_t * hydro, int iorformat_in,
			       int iorformat_out) {
  int nt[3];
  lgb_io_state_t * io[2];
  int rc = lgb_internal_hydro_io(hydro, nt, io, io + 1);
  if (rc) return rc;
  if (!fmt_valid(iorformat_in) || !fmt_valid(iorformat_out)) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "io record format");
  }
  for (int k = 0; k < 2; k++) {
    io[k]->fmt_in = iorformat_in;
    io[k]->fmt_out = iorformat_out;
  }
  return LUDWIG_GB_OK;
}

/* rho (1) then u (3) in one host array [4][nsites] */
static int hydro_io(hydro_t * hydro, int timestep, int write) {
  int nt[3];
  lgb_io_state_t * io[2];
  int rc = lgb_internal_hydro_io(hydro, nt, io, io + 1);
  if (rc) return rc;
  if (timestep < 0 || timestep >= 1000000000) {
    return lgb_internal_err(LUDWIG_GB_EINVAL, "hydro_io: timestep");
  }
  const long long n = (long long) nt[0]*nt[1]*nt[2];
  double * a = (double *) malloc((size_t) 4*n*sizeof(double));
  if (a == NULL) return lgb_internal_err(LUDWIG_GB_ENOMEM, "hydro io buffer");
  const char * stub[2] = {"rho", "vel"};
  const int nf[2] = {1, 3};
  double * part[2] = {a, a + n};
  if (write) rc = hydro_to_host(hydro, a, a + n, NULL);
  for (int k = 0; k < 2 && rc == 0; k++) {
    char file[256];
    data_name(file, sizeof(file), stub[k], timestep);
    if (write) {
      if (!io[k]->meta_written) {
	rc = write_metadata(stub[k], nt, io[k]->fmt_out, (io[k]->fmt_out ==
	     IO_RECORD_BINARY) ? nf[k] : nf[k]*ASCII_NBYTE + 1);
	if (rc == 0) io[k]->meta_written = 1;
      }
      if (rc == 0) rc = write_data(file, part[k], n, 1, nf[k], io[k]->fmt_out);
    }
    else {
      rc = read_data(file, part[k], n, 1, nf[k], io[k]->fmt_in);
    }
  }
  if (rc == 0 && !write) rc = hydro_from_host(hydro, a, a + n, NULL);
  free(a);
  return rc;
}

int hydro_io_write(hydro_t * hydro, int timestep, io_event_t * event) {
  (void) event;
  return hydro_io(hydro, timestep, 1);
}

int hydro_io_read(hydro_t * hydro, int timestep, io_event_t * event) {
  (void) event;
  return hydro_io(hydro, timestep, 0);
}
