/*
 * hoe_oracle.c — TEST INFRASTRUCTURE ONLY (the oracle; never the product).
 *
 * A plain-C FP64 restatement of the reference's CPU Array path of the
 * explicit higher-order encoding operator, used as the checker for the GPU
 * library and as the timed CPU baseline.  Only tests/, __graft_entry__.smoke()
 * and bench.py (cpu_baseline / --impl reference) may load it.
 *
 * Followed reference code (paths inside HighOrderMRI.jl):
 *   oracle_grid          src/Grid/Grid.jl:65-96 (r_j = (j-(N+1)/2)*delta, x fastest)
 *   oracle_basis         src/SphericalHarmonics/basisfunction.jl:27-126 (terms 1-17)
 *   oracle_forward       src/EncodingOperator/Explicit/array_operator.jl:241-288
 *                        (sample blocks of nSam/nBlock plus a remainder block,
 *                         phi = t*fieldmap + bf*kspha, e = exp(2*pi*i*phi),
 *                         out[p,:] = e*(x.*csm), out ./= sqrt(nVox))
 *   oracle_adjoint       array_operator.jl:294-348 (out += conj(e)*y[p,:],
 *                         ./sqrt(nVox), .*conj(csm), sum over coils)
 *   oracle_derivative    array_operator.jl:187-235 (e .* (bf*kspha_dt)' .* 2*pi*i)
 *   oracle_backward      no reference counterpart: analytic gradient of
 *                        0.5*||E x - y||^2 with respect to kspha, fieldmap, t0
 *
 * Layouts (Julia column-major, as in the C ABI): bf[v + l*nVox],
 * kspha[l + s*R], csm[2*(v + c*nVox)] (re, im), data y[2*(s + c*nSam)],
 * masked image xm[2*v].
 *
 * Build: oracle/Makefile (gcc -O2 -fopenmp, no fast-math).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define TWO_PI 6.283185307179586476925286766559

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Grid.jl:78-82: centred coordinates, x index fastest. */
void oracle_grid(int64_t nX, int64_t nY, int64_t nZ, double dx, double dy, double dz,
                 double *x, double *y, double *z) {
  for (int64_t k = 0; k < nZ; ++k)
    for (int64_t j = 0; j < nY; ++j)
      for (int64_t i = 0; i < nX; ++i) {
        int64_t o = i + nX * (j + nY * k);
        x[o] = ((double)(i + 1) - (double)(nX + 1) / 2.0) * dx;
        y[o] = ((double)(j + 1) - (double)(nY + 1) / 2.0) * dy;
        z[o] = ((double)(k + 1) - (double)(nZ + 1) / 2.0) * dz;
      }
}

/* One unnormalised real solid harmonic (1-based term index, 1..17).  Returns
 * 0 and writes *out, or -1 for an undefined term. */
static int basis_term(int term, double x, double y, double z, double *out) {
  double r2 = x * x + y * y + z * z;
  switch (term) {
    case 1: *out = 1.0; break;
    case 2: *out = x; break;
    case 3: *out = y; break;
    case 4: *out = z; break;
    case 5: *out = x * y; break;
    case 6: *out = z * y; break;
    case 7: *out = 3.0 * z * z - r2; break;
    case 8: *out = x * z; break;
    case 9: *out = x * x - y * y; break;
    case 10: *out = 3.0 * y * x * x - y * y * y; break;
    case 11: *out = x * z * y; break;
    case 12: *out = (5.0 * z * z - r2) * y; break;
    case 13: *out = 5.0 * z * z * z - 3.0 * z * r2; break;
    case 14: *out = (5.0 * z * z - r2) * x; break;
    case 15: *out = x * x * z - y * y * z; break;
    case 16: *out = x * x * x - 3.0 * x * y * y; break;
    case 17: *out = (x * y) * (x * x - y * y); break;
    default: return -1;
  }
  return 0;
}

/* basisfunction.jl:27-126: bf[v + idx*n] = term(terms[idx]). */
int oracle_basis(int64_t n, const double *x, const double *y, const double *z, int nterms,
                 const int *terms, double *bf) {
  for (int t = 0; t < nterms; ++t)
    for (int64_t v = 0; v < n; ++v)
      if (basis_term(terms[t], x[v], y[v], z[v], &bf[v + (int64_t)t * n]) != 0) return -1;
  return 0;
}

/* Sample partition of array_operator.jl:129-135: nBlock blocks of nSam/nBlock
 * samples and, if nSam % nBlock != 0, one remainder block. */
static int64_t block_bounds(int64_t nSam, int64_t nBlock, int64_t b, int64_t *lo, int64_t *hi) {
  if (nBlock > nSam) nBlock = nSam;
  int64_t n = nSam / nBlock;
  int64_t count = nBlock + ((nSam % nBlock) ? 1 : 0);
  if (b < nBlock) { *lo = n * b; *hi = n * (b + 1); }
  else { *lo = n * nBlock; *hi = nSam; }
  return count;
}

static double phase_of(int64_t s, int64_t v, int64_t nVox, int64_t R, const double *bf,
                       const double *kspha, const double *times, const double *fieldmap) {
  double ph = times[s] * (fieldmap ? fieldmap[v] : 0.0);
  for (int64_t l = 0; l < R; ++l) ph += bf[v + l * nVox] * kspha[l + s * R];
  return ph;
}

/* explicit_array_forward: y = E xm (masked image in), data layout samples fastest. */
void oracle_forward(int64_t nVox, int64_t nSam, int64_t nCha, int64_t R, const double *bf,
                    const double *kspha, const double *times, const double *fieldmap,
                    const double *csm, const double *xm, int64_t nBlock, double *y) {
  double *Z = (double *)malloc(sizeof(double) * 2 * nVox * nCha);
  for (int64_t c = 0; c < nCha; ++c)
    for (int64_t v = 0; v < nVox; ++v) {
      double xr = xm[2 * v], xi = xm[2 * v + 1];
      double cr = csm ? csm[2 * (v + c * nVox)] : 1.0, ci = csm ? csm[2 * (v + c * nVox) + 1] : 0.0;
      Z[2 * (v + c * nVox)] = xr * cr - xi * ci;
      Z[2 * (v + c * nVox) + 1] = xr * ci + xi * cr;
    }
  double scale = 1.0 / sqrt((double)nVox);
  int64_t lo, hi;
  int64_t nb = block_bounds(nSam, nBlock, 0, &lo, &hi);
  for (int64_t b = 0; b < nb; ++b) {
    block_bounds(nSam, nBlock, b, &lo, &hi);
#pragma omp parallel for schedule(static)
    for (int64_t s = lo; s < hi; ++s) {
      double *acc = (double *)calloc(2 * nCha, sizeof(double));
      for (int64_t v = 0; v < nVox; ++v) {
        double ph = phase_of(s, v, nVox, R, bf, kspha, times, fieldmap);
        double er = cos(TWO_PI * ph), ei = sin(TWO_PI * ph);
        for (int64_t c = 0; c < nCha; ++c) {
          double zr = Z[2 * (v + c * nVox)], zi = Z[2 * (v + c * nVox) + 1];
          acc[2 * c] += er * zr - ei * zi;
          acc[2 * c + 1] += er * zi + ei * zr;
        }
      }
      for (int64_t c = 0; c < nCha; ++c) {
        y[2 * (s + c * nSam)] = acc[2 * c] * scale;
        y[2 * (s + c * nSam) + 1] = acc[2 * c + 1] * scale;
      }
      free(acc);
    }
  }
  free(Z);
}

/* explicit_array_adjoint: xm = E^H y on the masked voxels. */
void oracle_adjoint(int64_t nVox, int64_t nSam, int64_t nCha, int64_t R, const double *bf,
                    const double *kspha, const double *times, const double *fieldmap,
                    const double *csm, const double *y, int64_t nBlock, double *xm) {
  double scale = 1.0 / sqrt((double)nVox);
  double *Q = (double *)calloc(2 * nVox * nCha, sizeof(double));
  int64_t lo, hi;
  int64_t nb = block_bounds(nSam, nBlock, 0, &lo, &hi);
  for (int64_t b = 0; b < nb; ++b) {
    block_bounds(nSam, nBlock, b, &lo, &hi);
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < nVox; ++v) {
      for (int64_t s = lo; s < hi; ++s) {
        double ph = phase_of(s, v, nVox, R, bf, kspha, times, fieldmap);
        double er = cos(TWO_PI * ph), ei = -sin(TWO_PI * ph); /* conj(e) */
        for (int64_t c = 0; c < nCha; ++c) {
          double yr = y[2 * (s + c * nSam)], yi = y[2 * (s + c * nSam) + 1];
          Q[2 * (v + c * nVox)] += er * yr - ei * yi;
          Q[2 * (v + c * nVox) + 1] += er * yi + ei * yr;
        }
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < nVox; ++v) {
    double sr = 0.0, si = 0.0;
    for (int64_t c = 0; c < nCha; ++c) {
      double qr = Q[2 * (v + c * nVox)] * scale, qi = Q[2 * (v + c * nVox) + 1] * scale;
      double cr = csm ? csm[2 * (v + c * nVox)] : 1.0, ci = csm ? -csm[2 * (v + c * nVox) + 1] : 0.0;
      sr += qr * cr - qi * ci;
      si += qr * ci + qi * cr;
    }
    xm[2 * v] = sr;
    xm[2 * v + 1] = si;
  }
  free(Q);
}

/* explicit_array_derivative: (B x)[s,c] with the factor 2*pi*i*(bf*kspha_dt)
 * over the nTerm spherical-harmonic rows (no fieldmap, no concomitant). */
void oracle_derivative(int64_t nVox, int64_t nSam, int64_t nCha, int64_t R, int64_t nTerm,
                       const double *bf, const double *kspha, const double *kspha_dt,
                       const double *times, const double *fieldmap, const double *csm,
                       const double *xm, double *y) {
  double scale = 1.0 / sqrt((double)nVox);
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < nSam; ++s) {
    double *acc = (double *)calloc(2 * nCha, sizeof(double));
    for (int64_t v = 0; v < nVox; ++v) {
      double ph = phase_of(s, v, nVox, R, bf, kspha, times, fieldmap);
      double g = 0.0;
      for (int64_t l = 0; l < nTerm; ++l) g += bf[v + l * nVox] * kspha_dt[l + s * nTerm];
      double er = cos(TWO_PI * ph), ei = sin(TWO_PI * ph);
      double fr = -TWO_PI * g * ei, fi = TWO_PI * g * er; /* e * 2*pi*i*g */
      for (int64_t c = 0; c < nCha; ++c) {
        double cr = csm ? csm[2 * (v + c * nVox)] : 1.0, ci = csm ? csm[2 * (v + c * nVox) + 1] : 0.0;
        double zr = xm[2 * v] * cr - xm[2 * v + 1] * ci, zi = xm[2 * v] * ci + xm[2 * v + 1] * cr;
        acc[2 * c] += fr * zr - fi * zi;
        acc[2 * c + 1] += fr * zi + fi * zr;
      }
    }
    for (int64_t c = 0; c < nCha; ++c) {
      y[2 * (s + c * nSam)] = acc[2 * c] * scale;
      y[2 * (s + c * nSam) + 1] = acc[2 * c + 1] * scale;
    }
    free(acc);
  }
}

/* Analytic gradient of L = 0.5*||E x - y||^2 given r = E x - y:
 *   G[s,v] = -(2 pi/sqrt(nVox)) Im(e^{i 2 pi phi} x_v sum_c conj(r[s,c]) csm[v,c])
 *   dk[l + s*R]  = sum_v G bf[v,l]
 *   ddf[v]       = sum_s G t_s
 *   dt0_b0       = -sum_{s,v} G fieldmap[v]
 *   dt0_coef     = -sum_{s,v} G sum_{l<nTerm} bf[v,l] kspha_dt[l,s]   (kspha_dt may be NULL) */
void oracle_backward(int64_t nVox, int64_t nSam, int64_t nCha, int64_t R, int64_t nTerm,
                     const double *bf, const double *kspha, const double *kspha_dt,
                     const double *times, const double *fieldmap, const double *csm,
                     const double *xm, const double *r, double *dk, double *ddf,
                     double *dt0_parts) {
  double sg = -TWO_PI / sqrt((double)nVox);
  double t0b = 0.0, t0c = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : t0b, t0c)
  for (int64_t s = 0; s < nSam; ++s) {
    for (int64_t l = 0; l < R; ++l) dk[l + s * R] = 0.0;
    for (int64_t v = 0; v < nVox; ++v) {
      double ph = phase_of(s, v, nVox, R, bf, kspha, times, fieldmap);
      double er = cos(TWO_PI * ph), ei = sin(TWO_PI * ph);
      double wr = 0.0, wi = 0.0;
      for (int64_t c = 0; c < nCha; ++c) {
        double cr = csm ? csm[2 * (v + c * nVox)] : 1.0, ci = csm ? csm[2 * (v + c * nVox) + 1] : 0.0;
        double rr = r[2 * (s + c * nSam)], ri = -r[2 * (s + c * nSam) + 1];
        wr += rr * cr - ri * ci;
        wi += rr * ci + ri * cr;
      }
      double xr = xm[2 * v], xi = xm[2 * v + 1];
      double pr = xr * wr - xi * wi, pi = xr * wi + xi * wr;       /* x_v * w */
      double G = sg * (er * pi + ei * pr);                         /* Im(e * p) */
      for (int64_t l = 0; l < R; ++l) dk[l + s * R] += G * bf[v + l * nVox];
      t0b -= G * (fieldmap ? fieldmap[v] : 0.0);
      if (kspha_dt) {
        double g = 0.0;
        for (int64_t l = 0; l < nTerm; ++l) g += bf[v + l * nVox] * kspha_dt[l + s * nTerm];
        t0c -= G * g;
      }
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t v = 0; v < nVox; ++v) {
    double acc = 0.0;
    for (int64_t s = 0; s < nSam; ++s) {
      double ph = phase_of(s, v, nVox, R, bf, kspha, times, fieldmap);
      double er = cos(TWO_PI * ph), ei = sin(TWO_PI * ph);
      double wr = 0.0, wi = 0.0;
      for (int64_t c = 0; c < nCha; ++c) {
        double cr = csm ? csm[2 * (v + c * nVox)] : 1.0, ci = csm ? csm[2 * (v + c * nVox) + 1] : 0.0;
        double rr = r[2 * (s + c * nSam)], ri = -r[2 * (s + c * nSam) + 1];
        wr += rr * cr - ri * ci;
        wi += rr * ci + ri * cr;
      }
      double xr = xm[2 * v], xi = xm[2 * v + 1];
      double pr = xr * wr - xi * wi, pi = xr * wi + xi * wr;
      acc += sg * (er * pi + ei * pr) * times[s];
    }
    ddf[v] = acc;
  }
  dt0_parts[0] = t0b;
  dt0_parts[1] = t0c;
}
