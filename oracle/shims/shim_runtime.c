/*
 * shim_runtime.c -- runtime behind the shim headers (mpi.h, fftw3.h,
 * fftw3-mpi.h, nanos6/debug.h) plus link stubs for the MFT_TAP solver
 * backend, which this build leaves out.  TEST INFRASTRUCTURE ONLY: linked
 * only into the reference build under oracle/_ref.
 */
#include <complex.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpi.h"
#include "fftw3.h"
#include "fftw3-mpi.h"
#include "nanos6/debug.h"
#include "../orc_fft.h"

/* ------------------------------------------------------------------ MPI */

typedef struct msg {
	int tag;
	size_t bytes;
	struct msg *next;
	unsigned char data[];
} msg_t;

static msg_t *q_head, *q_tail;

static size_t
type_size(MPI_Datatype t)
{
	switch(t)
	{
		case MPI_DOUBLE: return 8;
		case MPI_BYTE: return 1;
		case MPI_INT: return 4;
		case MPI_LONG: return 8;
		default: return 1;
	}
}

int MPI_Init(int *argc, char ***argv) { (void) argc; (void) argv; return MPI_SUCCESS; }

int
MPI_Init_thread(int *argc, char ***argv, int required, int *provided)
{
	(void) argc; (void) argv;
	if(provided) *provided = required;
	return MPI_SUCCESS;
}

int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void) c; *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void) c; *size = 1; return MPI_SUCCESS; }

int
MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm)
{
	size_t bytes = (size_t) count * type_size(type);
	msg_t *m = malloc(sizeof(msg_t) + bytes);
	(void) dest; (void) comm;
	if(!m) abort();
	m->tag = tag;
	m->bytes = bytes;
	m->next = NULL;
	memcpy(m->data, buf, bytes);
	if(q_tail) q_tail->next = m; else q_head = m;
	q_tail = m;
	return MPI_SUCCESS;
}

int
MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
		MPI_Request *req)
{
	static int token;
	int r = MPI_Send(buf, count, type, dest, tag, comm);
	if(req) *req = &token;
	return r;
}

int
MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
		MPI_Status *status)
{
	msg_t *m, *prev = NULL;
	size_t cap = (size_t) count * type_size(type);
	(void) src; (void) comm;
	for(m = q_head; m; prev = m, m = m->next)
		if(tag == MPI_ANY_TAG || m->tag == tag)
			break;
	if(!m)
	{
		fprintf(stderr, "mpi shim: receive with tag %d has no matching send on one rank\n", tag);
		abort();
	}
	memcpy(buf, m->data, m->bytes < cap ? m->bytes : cap);
	if(prev) prev->next = m->next; else q_head = m->next;
	if(q_tail == m) q_tail = prev;
	if(status) { status->MPI_SOURCE = 0; status->MPI_TAG = m->tag; status->MPI_ERROR = 0; }
	free(m);
	return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request *req, MPI_Status *status) { (void) status; if(req) *req = 0; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm c) { (void) c; return MPI_SUCCESS; }

int
MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm)
{
	(void) buf; (void) count; (void) type; (void) root; (void) comm;
	return MPI_SUCCESS;
}

int MPI_Abort(MPI_Comm c, int code) { (void) c; exit(code); }

/* ----------------------------------------------------------------- FFTW */

struct orc_fftw_plan {
	int r2c;
	int64_t n0, n1;       /* rows (y), columns (x) */
	double *real;         /* padded real array, row stride 2*(n1/2+1) */
	fftw_complex *cplx;   /* n0 x (n1/2+1) */
};

fftw_complex *fftw_alloc_complex(size_t n) { return malloc(sizeof(fftw_complex) * n); }
double *fftw_alloc_real(size_t n) { return malloc(sizeof(double) * n); }
void fftw_free(void *p) { free(p); }
void fftw_destroy_plan(fftw_plan p) { free(p); }
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int n) { (void) n; }
void fftw_mpi_init(void) {}

ptrdiff_t
fftw_mpi_local_size_2d(ptrdiff_t n0, ptrdiff_t n1, MPI_Comm comm, ptrdiff_t *local_n0,
		ptrdiff_t *local_0_start)
{
	(void) comm;
	*local_n0 = n0;
	*local_0_start = 0;
	return n0 * n1;
}

static fftw_plan
plan(int r2c, ptrdiff_t n0, ptrdiff_t n1, double *real, fftw_complex *cplx)
{
	fftw_plan p = calloc(1, sizeof(*p));
	if(!p) return NULL;
	p->r2c = r2c; p->n0 = n0; p->n1 = n1; p->real = real; p->cplx = cplx;
	return p;
}

fftw_plan
fftw_mpi_plan_dft_r2c_2d(ptrdiff_t n0, ptrdiff_t n1, double *in, fftw_complex *out, MPI_Comm comm,
		unsigned flags)
{
	(void) comm; (void) flags;
	return plan(1, n0, n1, in, out);
}

fftw_plan
fftw_mpi_plan_dft_c2r_2d(ptrdiff_t n0, ptrdiff_t n1, fftw_complex *in, double *out, MPI_Comm comm,
		unsigned flags)
{
	(void) comm; (void) flags;
	return plan(0, n0, n1, out, in);
}

/* Forward: rows then columns.  Inverse: columns then rows (unnormalised). */
void
fftw_execute(const fftw_plan p)
{
	int64_t nx = p->n1, ny = p->n0, nh = nx / 2 + 1, i;
	int64_t stride = 2 * nh;
	double *sr = malloc(sizeof(double) * (size_t) (nh * ny));
	double *si = malloc(sizeof(double) * (size_t) (nh * ny));
	if(p->r2c)
	{
		orc_rows_r2c(nx, ny, p->real, stride, sr, si);
		orc_cols(nx, ny, sr, si, -1);
		for(i = 0; i < nh * ny; i++)
		{
			/* C99 lays a double _Complex out as double[2] */
			((double *) &p->cplx[i])[0] = sr[i];
			((double *) &p->cplx[i])[1] = si[i];
		}
	}
	else
	{
		for(i = 0; i < nh * ny; i++) { sr[i] = creal(p->cplx[i]); si[i] = cimag(p->cplx[i]); }
		orc_cols(nx, ny, sr, si, +1);
		orc_rows_c2r(nx, ny, sr, si, p->real, stride);
	}
	free(sr); free(si);
}

/* --------------------------------------------------------------- others */

unsigned int nanos6_get_num_cpus(void) { return 1; }

/* The MFT_TAP backend (src/mft_tap.c, src/tap.c: MPI-3 shared windows and
 * MPI_Comm_spawn) is not built; selecting it fails cleanly. */
struct sim;
struct solver;
int MFT_TAP_init(struct sim *sim, struct solver *s)
{
	(void) sim; (void) s;
	fprintf(stderr, "MFT_TAP solver is not part of this build\n");
	return 1;
}
int MFT_TAP_solve(struct solver *s) { (void) s; return -1; }
int MFT_TAP_end(struct solver *s) { (void) s; return 0; }
