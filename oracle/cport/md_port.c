/*
 * md_port.c — C/OpenMP restatement of dompap's per-step loops, the timed
 * CPU baseline ("Numba-equivalent restatement", kind "port"). TEST AND
 * BENCHMARK INFRASTRUCTURE ONLY: never linked into the product.
 *
 * Each function follows the reference loop structure; loops the reference
 * runs under numba.prange are OpenMP-parallel here, loops it runs serially
 * stay serial:
 *   dp_port_nl_double_loop   dompap/neighbor_list.py:7-39     (prange over n)
 *   dp_port_nl_cell_list_3d  dompap/neighbor_list.py:106-180  (serial; its
 *                            cell width = cutoff, nc = ceil(L/cutoff) layout)
 *   dp_port_nl_is_old        dompap/neighbor_list.py:183-201  (serial)
 *   dp_port_forces           dompap/potential.py:163-188      (prange over n)
 *   dp_port_forces_types     the same with sigma/epsilon per type pair
 *   dp_port_gjf              dompap/integrator.py:17-40       (vectorised NumPy, serial)
 *   dp_port_wrap             dompap/positions.py:90-98        (NumPy, serial)
 * Arrays are row-major (N, D) float64 as in dompap. The pair force is a
 * function pointer f(r) (already cut at r_cut), like the reference's
 * first-class Numba closure.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double (*pair_fn)(double);

static inline double min_image(double d, double L) {
    if (d > L / 2) d -= L;
    else if (d < -L / 2) d += L;
    return d;
}

int dp_port_threads(void) {
#ifdef _OPENMP
    int n = 1;
#pragma omp parallel
    {
#pragma omp single
        n = omp_get_num_threads();
    }
    return n;
#else
    return 1;
#endif
}

/* returns the largest row length (rows longer than kmax are truncated) */
int64_t dp_port_nl_double_loop(const double *pos, int64_t n, int dim, const double *box, double cutoff, int kmax,
                               int32_t *nl) {
    int64_t maxc = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : maxc)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        int32_t *row = nl + i * kmax;
        for (int k = 0; k < kmax; ++k) row[k] = -1;
        for (int64_t j = 0; j < n; ++j) {
            if (i == j) continue;
            double q = 0.0;
            for (int d = 0; d < dim; ++d) {
                double x = min_image(pos[i * dim + d] - pos[j * dim + d], box[d]);
                q += x * x;
            }
            if (sqrt(q) < cutoff) {
                if (c < kmax) row[c] = (int32_t)j;
                ++c;
            }
        }
        if (c > maxc) maxc = c;
    }
    return maxc;
}

/* dompap's serial 3-D cell list, including its layout: cells of width
 * `cutoff`, nc = ceil(L / cutoff), capacity 27 * kmax per cell. */
int64_t dp_port_nl_cell_list_3d(const double *pos, int64_t n, const double *box, double cutoff, int kmax,
                                int32_t *nl) {
    int nc[3];
    for (int d = 0; d < 3; ++d) nc[d] = (int)ceil(box[d] / cutoff);
    const int64_t cap = (int64_t)kmax * 27;
    const int64_t ncell = (int64_t)nc[0] * nc[1] * nc[2];
    int32_t *cells = (int32_t *)malloc((size_t)(ncell * cap) * sizeof(int32_t));
    int32_t *fill = (int32_t *)calloc((size_t)ncell, sizeof(int32_t));
    if (!cells || !fill) {
        free(cells);
        free(fill);
        return -1;
    }
    for (int64_t t = 0; t < ncell * cap; ++t) cells[t] = -1;
    for (int64_t i = 0; i < n; ++i) {
        int c[3];
        for (int d = 0; d < 3; ++d) {
            c[d] = (int)floor(pos[i * 3 + d] / cutoff);
            if (c[d] < 0) c[d] = 0;
            if (c[d] >= nc[d]) c[d] = nc[d] - 1;
        }
        const int64_t l = ((int64_t)c[0] * nc[1] + c[1]) * nc[2] + c[2];
        /* the reference counts the occupied slots (np.sum(cell != -1)) */
        int64_t idx = 0;
        for (int64_t s = 0; s < cap; ++s) idx += cells[l * cap + s] != -1;
        if (idx < cap) cells[l * cap + idx] = (int32_t)i;
        fill[l] = (int32_t)(idx + 1);
    }
    int64_t maxc = 0;
    for (int64_t i = 0; i < n; ++i) {
        int64_t cnt = 0;
        int32_t *row = nl + i * kmax;
        for (int k = 0; k < kmax; ++k) row[k] = -1;
        int c[3];
        for (int d = 0; d < 3; ++d) {
            c[d] = (int)floor(pos[i * 3 + d] / cutoff);
            if (c[d] < 0) c[d] = 0;
            if (c[d] >= nc[d]) c[d] = nc[d] - 1;
        }
        for (int s = 0; s < 27; ++s) {
            int cc[3], tmp = s;
            for (int d = 0; d < 3; ++d) {
                cc[d] = c[d] + tmp % 3 - 1;
                tmp /= 3;
                if (cc[d] < 0) cc[d] += nc[d];
                else if (cc[d] >= nc[d]) cc[d] -= nc[d];
            }
            const int64_t l = ((int64_t)cc[0] * nc[1] + cc[1]) * nc[2] + cc[2];
            for (int64_t m = 0; m < cap; ++m) {
                const int32_t j = cells[l * cap + m];
                if (j == -1) break;
                double q = 0.0;
                for (int d = 0; d < 3; ++d) {
                    double x = min_image(pos[i * 3 + d] - pos[(int64_t)j * 3 + d], box[d]);
                    q += x * x;
                }
                if (sqrt(q) < cutoff && j != i) {
                    if (cnt < kmax) row[cnt] = j;
                    ++cnt;
                }
            }
        }
        if (cnt > maxc) maxc = cnt;
    }
    free(cells);
    free(fill);
    return maxc;
}

int dp_port_nl_is_old(const double *pos, const double *ref, int64_t n, int dim, const double *box, double skin) {
    double maxq = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double q = 0.0;
        for (int d = 0; d < dim; ++d) {
            double x = min_image(pos[i * dim + d] - ref[i * dim + d], box[d]);
            q += x * x;
        }
        if (q > maxq) maxq = q;
    }
    return maxq > (0.5 * skin) * (0.5 * skin);
}

void dp_port_forces(const double *pos, int64_t n, int dim, const double *box, const int32_t *nl, int kmax,
                    pair_fn f, double sigma, double epsilon, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int k = 0; k < kmax; ++k) {
            const int32_t j = nl[i * kmax + k];
            if (j == -1) break;
            double d[8], q = 0.0;
            for (int c = 0; c < dim; ++c) {
                d[c] = min_image(pos[i * dim + c] - pos[(int64_t)j * dim + c], box[c]);
                q += d[c] * d[c];
            }
            const double r = sqrt(q);
            const double sf = epsilon * f(r / sigma);
            for (int c = 0; c < dim; ++c) acc[c] = acc[c] + sf * (d[c] / r);
        }
        for (int c = 0; c < dim; ++c) out[i * dim + c] = acc[c];
    }
}

/* dp_port_forces with sigma(n, m), epsilon(n, m) from per-type tables
 * (dompap/potential.py:163-188 calling its index callables sigma_func(n, m),
 * epsilon_func(n, m), which the binary-mixture example makes table lookups by
 * particle type: examples/wahnstrom_mixture.py:52-63). */
void dp_port_forces_types(const double *pos, int64_t n, int dim, const double *box, const int32_t *nl, int kmax,
                          pair_fn f, const int32_t *types, int ntypes, const double *sig_tab,
                          const double *eps_tab, double *out) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int ti = types[i];
        for (int k = 0; k < kmax; ++k) {
            const int32_t j = nl[i * kmax + k];
            if (j == -1) break;
            double d[8], q = 0.0;
            for (int c = 0; c < dim; ++c) {
                d[c] = min_image(pos[i * dim + c] - pos[(int64_t)j * dim + c], box[c]);
                q += d[c] * d[c];
            }
            const double r = sqrt(q);
            const int p = ti * ntypes + types[j];
            const double sf = eps_tab[p] * f(r / sig_tab[p]);
            for (int c = 0; c < dim; ++c) acc[c] = acc[c] + sf * (d[c] / r);
        }
        for (int c = 0; c < dim; ++c) out[i * dim + c] = acc[c];
    }
}

/* xoshiro256** + Box-Muller standard normals (the reference draws
 * np.random.normal inside its step, serially). */
static uint64_t rng_s[4] = {0x9E3779B97F4A7C15ull, 0xBF58476D1CE4E5B9ull, 0x94D049BB133111EBull, 0x2545F4914F6CDD1Dull};
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint64_t xnext(void) {
    const uint64_t r = rotl(rng_s[1] * 5, 7) * 9, t = rng_s[1] << 17;
    rng_s[2] ^= rng_s[0];
    rng_s[3] ^= rng_s[1];
    rng_s[1] ^= rng_s[2];
    rng_s[0] ^= rng_s[3];
    rng_s[2] ^= t;
    rng_s[3] = rotl(rng_s[3], 45);
    return r;
}
void dp_port_seed(uint64_t seed) {
    for (int k = 0; k < 4; ++k) {
        seed += 0x9E3779B97F4A7C15ull;
        uint64_t z = seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        rng_s[k] = z ^ (z >> 31);
    }
}
void dp_port_normals(double *z, int64_t count) {
    for (int64_t t = 0; t < count; t += 2) {
        const double u = ((double)(xnext() >> 11) + 1.0) * (1.0 / 9007199254740992.0);
        const double v = (double)(xnext() >> 11) * (1.0 / 9007199254740992.0);
        const double rad = sqrt(-2.0 * log(u));
        z[t] = rad * cos(6.283185307179586 * v);
        if (t + 1 < count) z[t + 1] = rad * sin(6.283185307179586 * v);
    }
}

void dp_port_gjf(double *pos, double *vel, double *beta, const double *force, const double *mass, int64_t n, int dim,
                 double dt, double temperature, double tau, double *scratch) {
    dp_port_normals(scratch, n * dim);
    for (int64_t i = 0; i < n; ++i) {
        const double m = mass[i];
        const double alpha = m / tau;
        const double beta_variance = 2 * alpha * temperature * dt;
        const double numerator = 1.0 - alpha * dt / 2.0 / m;
        const double denominator = 1.0 + alpha * dt / 2.0 / m;
        const double a = numerator / denominator;
        const double b = 1 / denominator;
        for (int d = 0; d < dim; ++d) {
            const int64_t o = i * dim + d;
            const double bn = sqrt(beta_variance) * scratch[o];
            vel[o] = a * vel[o] + b * dt * force[o] / m + b * (beta[o] + bn) / 2 / m;
            pos[o] = pos[o] + vel[o] * dt;
            beta[o] = bn;
        }
    }
}

void dp_port_wrap(double *pos, int32_t *img, int64_t n, int dim, const double *box) {
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < dim; ++d) {
            const int64_t o = i * dim + d;
            const double s = floor(pos[o] / box[d]);
            img[o] += (int32_t)s;
            pos[o] -= s * box[d];
        }
}
