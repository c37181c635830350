/*
 * orc_fft.h -- the FP64 FFT of the oracle, shared by the C restatement
 * (cpic_oracle.c) and by the FFTW-API shim that the reference's own
 * solver.c is compiled against (shims/shim_runtime.c).  Both therefore
 * transform identically: the reference build and the restatement give the
 * same phi for the same rho.  TEST INFRASTRUCTURE ONLY.
 *
 * orc_fft1: in-place iterative radix-2 complex transform, sign -1 forward,
 * +1 inverse, unnormalised; n a power of two, else a direct DFT.
 * orc_rows_r2c / orc_cols / orc_rows_c2r: the passes of a 2D real
 * transform of ny rows x nx columns with FFTW's half-spectrum layout
 * (ny x (nx/2+1) complex).
 */
#ifndef ORC_FFT_H
#define ORC_FFT_H

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void
orc_fft1(double *re, double *im, int64_t n, int sign)
{
	int64_t i, j, k, len;
	if(n <= 1) return;
	if(n & (n - 1))
	{
		double *tr = malloc(sizeof(double) * (size_t) n);
		double *ti = malloc(sizeof(double) * (size_t) n);
		for(k = 0; k < n; k++)
		{
			double sr = 0.0, si = 0.0;
			for(j = 0; j < n; j++)
			{
				double a = sign * 2.0 * M_PI * (double) ((k * j) % n) / (double) n;
				double c = cos(a), s = sin(a);
				sr += re[j] * c - im[j] * s;
				si += re[j] * s + im[j] * c;
			}
			tr[k] = sr; ti[k] = si;
		}
		memcpy(re, tr, sizeof(double) * (size_t) n);
		memcpy(im, ti, sizeof(double) * (size_t) n);
		free(tr); free(ti);
		return;
	}
	for(i = 1, j = 0; i < n; i++)
	{
		int64_t bit = n >> 1;
		for(; j & bit; bit >>= 1) j ^= bit;
		j ^= bit;
		if(i < j)
		{
			double t = re[i]; re[i] = re[j]; re[j] = t;
			t = im[i]; im[i] = im[j]; im[j] = t;
		}
	}
	for(len = 2; len <= n; len <<= 1)
	{
		int64_t half = len >> 1;
		for(k = 0; k < half; k++)
		{
			double a = sign * 2.0 * M_PI * (double) k / (double) len;
			double wr = cos(a), wi = sin(a);
			for(i = k; i < n; i += len)
			{
				int64_t p = i + half;
				double xr = re[p] * wr - im[p] * wi;
				double xi = re[p] * wi + im[p] * wr;
				re[p] = re[i] - xr; im[p] = im[i] - xi;
				re[i] = re[i] + xr; im[i] = im[i] + xi;
			}
		}
	}
}

/* Real rows (row stride rstride) -> half spectra sr/si (row stride nx/2+1). */
static void
orc_rows_r2c(int64_t nx, int64_t ny, const double *in, int64_t rstride, double *sr, double *si)
{
	int64_t ix, iy, nh = nx / 2 + 1;
	double *br = malloc(sizeof(double) * (size_t) nx);
	double *bi = malloc(sizeof(double) * (size_t) nx);
	for(iy = 0; iy < ny; iy++)
	{
		for(ix = 0; ix < nx; ix++) { br[ix] = in[iy * rstride + ix]; bi[ix] = 0.0; }
		orc_fft1(br, bi, nx, -1);
		for(ix = 0; ix < nh; ix++) { sr[iy * nh + ix] = br[ix]; si[iy * nh + ix] = bi[ix]; }
	}
	free(br); free(bi);
}

/* Transform every spectrum column along y (sign as orc_fft1). */
static void
orc_cols(int64_t nx, int64_t ny, double *sr, double *si, int sign)
{
	int64_t ix, iy, nh = nx / 2 + 1;
	double *br = malloc(sizeof(double) * (size_t) ny);
	double *bi = malloc(sizeof(double) * (size_t) ny);
	for(ix = 0; ix < nh; ix++)
	{
		for(iy = 0; iy < ny; iy++) { br[iy] = sr[iy * nh + ix]; bi[iy] = si[iy * nh + ix]; }
		orc_fft1(br, bi, ny, sign);
		for(iy = 0; iy < ny; iy++) { sr[iy * nh + ix] = br[iy]; si[iy * nh + ix] = bi[iy]; }
	}
	free(br); free(bi);
}

/* Half spectra -> real rows, unnormalised, as a c2r transform: each row
 * is Hermitian-extended (X[nx-k] = conj(X[k])) with the imaginary parts of
 * the DC and Nyquist bins ignored. */
static void
orc_rows_c2r(int64_t nx, int64_t ny, const double *sr, const double *si, double *out,
		int64_t ostride)
{
	int64_t ix, iy, nh = nx / 2 + 1;
	double *br = malloc(sizeof(double) * (size_t) nx);
	double *bi = malloc(sizeof(double) * (size_t) nx);
	for(iy = 0; iy < ny; iy++)
	{
		for(ix = 0; ix < nh; ix++) { br[ix] = sr[iy * nh + ix]; bi[ix] = si[iy * nh + ix]; }
		bi[0] = 0.0;
		if(nx % 2 == 0) bi[nx / 2] = 0.0;
		for(ix = nh; ix < nx; ix++) { br[ix] = br[nx - ix]; bi[ix] = -bi[nx - ix]; }
		orc_fft1(br, bi, nx, +1);
		for(ix = 0; ix < nx; ix++) out[iy * ostride + ix] = br[ix];
	}
	free(br); free(bi);
}

#endif /* ORC_FFT_H */
