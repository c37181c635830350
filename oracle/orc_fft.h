/*
 * orc_fft.h -- the FP64 FFT of the oracle, shared by the C restatement
 * (cpic_oracle.c) and by the FFTW-API shim that the reference's own
 * solver.c is compiled against (shims/shim_runtime.c).  Both therefore
 * transform identically: the reference build and the restatement give the
 * same phi for the same rho.  TEST INFRASTRUCTURE ONLY.
 *
 * orc_fft1: in-place complex transform, sign -1 forward, +1 inverse,
 * unnormalised: iterative radix-2 for n a power of two, else a recursive
 * mixed-radix decimation in time (Cooley-Tukey) over the prime factors of
 * n, prime lengths summed directly.
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

/* Twiddle tables exp(sign 2 pi i j / n), j < n, of the lengths that are
 * not powers of two (a 2D transform uses four: both sides, both signs). */
struct orc_tw { int64_t n; int sign; double *c, *s; };
static struct orc_tw orc_tw_cache[4];
static int orc_tw_next;

static const struct orc_tw *
orc_twiddles(int64_t n, int sign)
{
	int k;
	int64_t j;
	struct orc_tw *t;
	for(k = 0; k < 4; k++)
		if(orc_tw_cache[k].c && orc_tw_cache[k].n == n && orc_tw_cache[k].sign == sign)
			return &orc_tw_cache[k];
	t = &orc_tw_cache[orc_tw_next];
	orc_tw_next = (orc_tw_next + 1) % 4;
	free(t->c);
	free(t->s);
	t->n = n;
	t->sign = sign;
	t->c = malloc(sizeof(double) * (size_t) n);
	t->s = malloc(sizeof(double) * (size_t) n);
	for(j = 0; j < n; j++)
	{
		double a = sign * 2.0 * M_PI * (double) j / (double) n;
		t->c[j] = cos(a);
		t->s[j] = sin(a);
	}
	return t;
}

static int64_t
orc_smallest_factor(int64_t n)
{
	int64_t p;
	if(n % 2 == 0) return 2;
	for(p = 3; p * p <= n; p += 2)
		if(n % p == 0) return p;
	return n;
}

/* Length-n transform in place by decimation in time: with p the smallest
 * prime factor of n and m = n / p, the subsequences x[r], x[r + p], ...
 * (r < p) are transformed at length m and combined as
 * X[k] = sum_r W_n^(r k) Y_r[k mod m]; a prime length is summed directly.
 * W_n^j is read from the table of the top length N (index j N / n); tr, ti
 * hold n values of scratch, free whenever a sub-transform runs. */
static void
orc_mixed(double *re, double *im, int64_t n, const struct orc_tw *tw, double *tr, double *ti)
{
	int64_t p, m, step, r, j, k;
	if(n <= 1) return;
	p = orc_smallest_factor(n);
	m = n / p;
	step = tw->n / n;
	if(p < n)
	{
		for(r = 0; r < p; r++)
			for(j = 0; j < m; j++)
			{
				tr[r * m + j] = re[j * p + r];
				ti[r * m + j] = im[j * p + r];
			}
		memcpy(re, tr, sizeof(double) * (size_t) n);
		memcpy(im, ti, sizeof(double) * (size_t) n);
		for(r = 0; r < p; r++)
			orc_mixed(re + r * m, im + r * m, m, tw, tr, ti);
	}
	for(k = 0; k < n; k++)
	{
		double sr = 0.0, si = 0.0;
		for(r = 0; r < p; r++)
		{
			/* p == n: r runs over the samples and Y_r[0] = x[r] */
			const int64_t y = r * m + k % m;
			const int64_t w = ((r * k) % n) * step;
			sr += re[y] * tw->c[w] - im[y] * tw->s[w];
			si += re[y] * tw->s[w] + im[y] * tw->c[w];
		}
		tr[k] = sr;
		ti[k] = si;
	}
	memcpy(re, tr, sizeof(double) * (size_t) n);
	memcpy(im, ti, sizeof(double) * (size_t) n);
}

static void
orc_fft1(double *re, double *im, int64_t n, int sign)
{
	int64_t i, j, k, len;
	if(n <= 1) return;
	if(n & (n - 1))
	{
		const struct orc_tw *tw = orc_twiddles(n, sign);
		double *tr = malloc(sizeof(double) * (size_t) n);
		double *ti = malloc(sizeof(double) * (size_t) n);
		orc_mixed(re, im, n, tw, tr, ti);
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
