/*
 * qf_oracle.c — CPU oracle (TEST INFRASTRUCTURE, not product code).
 *
 * A plain-C restatement of QuantumForge's complex128 CPU state-vector
 * simulator, used only by the test-suite, the smoke check and the CPU leg of
 * the benchmark. Every function names the reference file:line it follows.
 * Build with -ffp-contract=off (see oracle/Makefile): Rust never contracts
 * a*b+c into an FMA, and neither may this file.
 */
#include "qf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- Complex64 (src/lib.rs:437-505) ------------------------------------ */
typedef struct { double re, im; } cplx;

static inline cplx c_new(double re, double im) { cplx c = {re, im}; return c; }
static inline cplx c_add(cplx a, cplx b) { return c_new(a.re + b.re, a.im + b.im); }
/* impl Mul for Complex64: (ar*br - ai*bi, ar*bi + ai*br), src/lib.rs:485-493 */
static inline cplx c_mul(cplx a, cplx b) {
    return c_new(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
static inline cplx c_mulf(cplx a, double s) { return c_new(a.re * s, a.im * s); }
static inline cplx c_divf(cplx a, double s) { return c_new(a.re / s, a.im / s); }
static inline cplx c_conj(cplx a) { return c_new(a.re, -a.im); }
static inline double c_norm_sqr(cplx a) { return a.re * a.re + a.im * a.im; }

#define AMP(p, i) (((cplx *)(p))[(i)])

/* Rust's `impl Sum for f64` folds from -0.0 (std, since 1.83). */
#define SUM_INIT (-0.0)

/* ---- SmallRng (src/lib.rs:4881-4911) ----------------------------------- */
uint64_t qfo_rng_seeded(uint64_t seed) {
    uint64_t z = seed + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    return z == 0 ? 0x9E3779B97F4A7C15ULL : z;
}

uint64_t qfo_rng_next_u64(uint64_t *state) {
    uint64_t x = *state;
    x ^= x << 13;
    x ^= x >> 7;
    x ^= x << 17;
    *state = x;
    return x;
}

double qfo_rng_next_f64(uint64_t *state) {
    return (double)(qfo_rng_next_u64(state) >> 11) * (1.0 / (double)(1ULL << 53));
}

/* ---- Gate::matrix (src/lib.rs:2267-2333) ------------------------------- */
static int gate_matrix(int gate, double theta, cplx m[4]) {
    const cplx z = c_new(0.0, 0.0), o = c_new(1.0, 0.0), i = c_new(0.0, 1.0);
    const double s = 0.70710678118654752440; /* FRAC_1_SQRT_2 */
    switch (gate) {
    case QF_GATE_I: m[0] = o; m[1] = z; m[2] = z; m[3] = o; return 0;
    case QF_GATE_X: m[0] = z; m[1] = o; m[2] = o; m[3] = z; return 0;
    case QF_GATE_Y: m[0] = z; m[1] = c_new(0.0, -1.0); m[2] = i; m[3] = z; return 0;
    case QF_GATE_Z: m[0] = o; m[1] = z; m[2] = z; m[3] = c_new(-1.0, 0.0); return 0;
    case QF_GATE_H:
        m[0] = c_new(s, 0.0); m[1] = c_new(s, 0.0); m[2] = c_new(s, 0.0); m[3] = c_new(-s, 0.0);
        return 0;
    case QF_GATE_S: m[0] = o; m[1] = z; m[2] = z; m[3] = i; return 0;
    case QF_GATE_SDG: m[0] = o; m[1] = z; m[2] = z; m[3] = c_new(0.0, -1.0); return 0;
    case QF_GATE_T: m[0] = o; m[1] = z; m[2] = z; m[3] = c_new(s, s); return 0;
    case QF_GATE_TDG: m[0] = o; m[1] = z; m[2] = z; m[3] = c_new(s, -s); return 0;
    case QF_GATE_RX: {
        double c = cos(theta * 0.5), si = sin(theta * 0.5);
        m[0] = c_new(c, 0.0); m[1] = c_new(0.0, -si); m[2] = c_new(0.0, -si); m[3] = c_new(c, 0.0);
        return 0;
    }
    case QF_GATE_RY: {
        double c = cos(theta * 0.5), si = sin(theta * 0.5);
        m[0] = c_new(c, 0.0); m[1] = c_new(-si, 0.0); m[2] = c_new(si, 0.0); m[3] = c_new(c, 0.0);
        return 0;
    }
    case QF_GATE_RZ: {
        double half = theta * 0.5;
        m[0] = c_new(cos(half), -sin(half)); m[1] = z; m[2] = z; m[3] = c_new(cos(half), sin(half));
        return 0;
    }
    default: return QF_ERR_INVALID_ARGUMENT;
    }
}

int qfo_gate_matrix(int gate, double theta, double out[8]) {
    cplx m[4];
    int st = gate_matrix(gate, theta, m);
    if (st) return st;
    for (int k = 0; k < 4; ++k) { out[2 * k] = m[k].re; out[2 * k + 1] = m[k].im; }
    return 0;
}

/* rotation_gate (src/lib.rs:2355-2361): axis X/Y/Z -> Rx/Ry/Rz. */
static int rotation_gate(int axis) {
    return axis == QF_PAULI_X ? QF_GATE_RX : axis == QF_PAULI_Y ? QF_GATE_RY : QF_GATE_RZ;
}

/* adjoint_gate (src/lib.rs:2363-2382). */
static void adjoint_gate(int gate, double theta, int *g_out, double *t_out) {
    *t_out = theta;
    switch (gate) {
    case QF_GATE_RX: case QF_GATE_RY: case QF_GATE_RZ: *g_out = gate; *t_out = -theta; return;
    case QF_GATE_S: *g_out = QF_GATE_SDG; return;
    case QF_GATE_SDG: *g_out = QF_GATE_S; return;
    case QF_GATE_T: *g_out = QF_GATE_TDG; return;
    case QF_GATE_TDG: *g_out = QF_GATE_T; return;
    default: *g_out = gate; return;
    }
}

/* ---- StateVector (src/lib.rs:928-1351) --------------------------------- */
int qfo_sv_zero(double *amps, uint32_t n) {
    if (n == 0) return QF_ERR_ZERO_QUBITS;
    uint64_t dim = 1ULL << n;
    memset(amps, 0, sizeof(double) * 2 * dim);
    amps[0] = 1.0;
    return 0;
}

/* StateVector::apply (src/lib.rs:1017-1059). threads == 0 is the sequential
 * branch (:1046-1057); threads > 0 restates the rayon branch (:1027-1044):
 * clone the whole vector, map every index in parallel into a fresh buffer,
 * replace. Both produce the same values: new0 = m00*a0 + m01*a1,
 * new1 = m10*a0 + m11*a1. */
int qfo_sv_apply(double *amps, uint32_t n, int gate, double theta, uint32_t target, int threads) {
    if (target >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    cplx m[4];
    int st = gate_matrix(gate, theta, m);
    if (st) return st;
    const uint64_t mask = 1ULL << target, dim = 1ULL << n;
    cplx *a = (cplx *)amps;
    if (threads <= 0) {
        for (uint64_t base = 0; base < dim; ++base) {
            if ((base & mask) == 0) {
                cplx a0 = a[base], a1 = a[base | mask];
                a[base] = c_add(c_mul(m[0], a0), c_mul(m[1], a1));
                a[base | mask] = c_add(c_mul(m[2], a0), c_mul(m[3], a1));
            }
        }
        return 0;
    }
    cplx *old = (cplx *)malloc(sizeof(cplx) * dim);
    cplx *nw = (cplx *)malloc(sizeof(cplx) * dim);
    if (!old || !nw) { free(old); free(nw); return QF_ERR_MEMORY_ALLOCATION_FAILED; }
    int64_t sdim = (int64_t)dim;
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < sdim; ++i) old[i] = a[i];
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < sdim; ++i) {
        uint64_t idx = (uint64_t)i;
        if ((idx & mask) == 0) nw[idx] = c_add(c_mul(m[0], old[idx]), c_mul(m[1], old[idx | mask]));
        else nw[idx] = c_add(c_mul(m[2], old[idx & ~mask]), c_mul(m[3], old[idx]));
    }
#pragma omp parallel for num_threads(threads) schedule(static)
    for (int64_t i = 0; i < sdim; ++i) a[i] = nw[i];
    free(old);
    free(nw);
    return 0;
}

/* StateVector::check_pair (src/lib.rs:1124-1142). */
static int check_pair(uint32_t n, uint32_t first, uint32_t second) {
    if (first >= n || second >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    if (first == second) return QF_ERR_INVALID_QUBIT_PAIR;
    return 0;
}

/* StateVector::apply_cnot (src/lib.rs:1062-1080): swap (c=1,t=0) <-> (c=1,t=1). */
int qfo_sv_apply_cnot(double *amps, uint32_t n, uint32_t control, uint32_t target) {
    int st = check_pair(n, control, target);
    if (st) return st;
    const uint64_t cm = 1ULL << control, tm = 1ULL << target, dim = 1ULL << n;
    cplx *a = (cplx *)amps;
    for (uint64_t i = 0; i < dim; ++i) {
        if ((i & cm) && !(i & tm)) { cplx t = a[i]; a[i] = a[i | tm]; a[i | tm] = t; }
    }
    return 0;
}

/* StateVector::apply_cz (src/lib.rs:1083-1101): amplitude * -1.0 where both bits are 1. */
int qfo_sv_apply_cz(double *amps, uint32_t n, uint32_t first, uint32_t second) {
    int st = check_pair(n, first, second);
    if (st) return st;
    const uint64_t both = (1ULL << first) | (1ULL << second), dim = 1ULL << n;
    cplx *a = (cplx *)amps;
    for (uint64_t i = 0; i < dim; ++i)
        if ((i & both) == both) a[i] = c_mulf(a[i], -1.0);
    return 0;
}

/* StateVector::apply_swap (src/lib.rs:1104-1122): exchange 01 <-> 10. */
int qfo_sv_apply_swap(double *amps, uint32_t n, uint32_t first, uint32_t second) {
    int st = check_pair(n, first, second);
    if (st) return st;
    const uint64_t fm = 1ULL << first, sm = 1ULL << second, dim = 1ULL << n;
    cplx *a = (cplx *)amps;
    for (uint64_t i = 0; i < dim; ++i) {
        if ((i & sm) && !(i & fm)) {
            uint64_t j = i ^ fm ^ sm;
            cplx t = a[i]; a[i] = a[j]; a[j] = t;
        }
    }
    return 0;
}

/* StateVector::norm_sqr (src/lib.rs:998-1000). */
double qfo_sv_norm_sqr(const double *amps, uint32_t n) {
    const uint64_t dim = 1ULL << n;
    double s = SUM_INIT;
    for (uint64_t i = 0; i < dim; ++i) s += c_norm_sqr(AMP(amps, i));
    return s;
}

/* StateVector::probabilities (src/lib.rs:1144-1146). */
void qfo_sv_probabilities(const double *amps, uint32_t n, double *out) {
    const uint64_t dim = 1ULL << n;
    for (uint64_t i = 0; i < dim; ++i) out[i] = c_norm_sqr(AMP(amps, i));
}

/* expectation_z / _x / _y (src/lib.rs:1149-1166, 1278-1302), dispatch :1304-1318. */
int qfo_sv_expectation(const double *amps, uint32_t n, int observable, uint32_t qubit, double *out) {
    if (qubit >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    const uint64_t mask = 1ULL << qubit, dim = 1ULL << n;
    double s = SUM_INIT;
    if (observable == QF_PAULI_Z) {
        for (uint64_t i = 0; i < dim; ++i) {
            double sign = (i & mask) == 0 ? 1.0 : -1.0;
            s += sign * c_norm_sqr(AMP(amps, i));
        }
    } else if (observable == QF_PAULI_X || observable == QF_PAULI_Y) {
        for (uint64_t i = 0; i < dim; ++i) {
            if (i & mask) continue;
            cplx p = c_mul(c_conj(AMP(amps, i)), AMP(amps, i | mask));
            s += (observable == QF_PAULI_X ? p.re : p.im) * 2.0;
        }
    } else {
        return QF_ERR_INVALID_ARGUMENT;
    }
    *out = s;
    return 0;
}

/* StateVector::measure (src/lib.rs:1321-1351). */
int qfo_sv_measure(double *amps, uint32_t n, uint32_t qubit, uint64_t *rng_state, uint8_t *outcome) {
    if (qubit >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    const uint64_t mask = 1ULL << qubit, dim = 1ULL << n;
    cplx *a = (cplx *)amps;
    double p_one = SUM_INIT;
    for (uint64_t i = 0; i < dim; ++i)
        if (i & mask) p_one += c_norm_sqr(a[i]);
    /* f64::clamp(0.0, 1.0) */
    if (p_one < 0.0) p_one = 0.0;
    if (p_one > 1.0) p_one = 1.0;
    uint8_t o = qfo_rng_next_f64(rng_state) < p_one ? 1 : 0;
    double probability = o == 1 ? p_one : 1.0 - p_one;
    if (probability <= DBL_EPSILON) return QF_ERR_INVALID_PROBABILITY;
    double scale = sqrt(probability);
    for (uint64_t i = 0; i < dim; ++i) {
        if ((uint8_t)((i & mask) != 0) != o) a[i] = c_new(0.0, 0.0);
        else a[i] = c_divf(a[i], scale);
    }
    *outcome = o;
    return 0;
}

/* StateVector::normalize (src/lib.rs:1005-1014): divide by sqrt(norm_sqr). */
int qfo_sv_normalize(double *amps, uint32_t n) {
    const double norm = sqrt(qfo_sv_norm_sqr(amps, n));
    if (norm == 0.0 || !isfinite(norm)) return QF_ERR_INVALID_PROBABILITY;
    cplx *a = (cplx *)amps;
    const uint64_t dim = 1ULL << n;
    for (uint64_t i = 0; i < dim; ++i) a[i] = c_divf(a[i], norm);
    return 0;
}

/* validate_probability (src/lib.rs:2229-2235). */
static int valid_probability(double p) { return isfinite(p) && p >= 0.0 && p <= 1.0; }

/* Sequential index-order sum of norm_sqr over the amplitudes whose `mask` bit
 * is set (the probability_one of src/lib.rs:1390-1396 and :1449-1455). */
static double p_one_sum(const cplx *a, uint64_t dim, uint64_t mask) {
    double s = SUM_INIT;
    for (uint64_t i = 0; i < dim; ++i)
        if (i & mask) s += c_norm_sqr(a[i]);
    return s;
}

static double clamp01(double x) { return x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x); }

/* StateVector::apply_channel_trajectory (src/lib.rs:1356-1506): one uniform
 * from the shot's stream selects a Kraus branch, which is applied and
 * renormalised. Thermal rates follow NoiseChannel::thermal_rates
 * (src/lib.rs:1611-1626): gamma_up = gamma_down * exp(-beta_delta). */
int qfo_sv_channel_trajectory(double *amps, uint32_t n, int channel, double p, double beta_delta, uint32_t qubit,
                              uint64_t *rng_state) {
    if (qubit >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    cplx *a = (cplx *)amps;
    const uint64_t mask = 1ULL << qubit, dim = 1ULL << n;
    if (channel == QF_CHANNEL_DEPOLARIZING) {
        if (!valid_probability(p)) return QF_ERR_INVALID_PROBABILITY;
        const double sample = qfo_rng_next_f64(rng_state);
        if (sample >= 1.0 - p && p > 0.0) {
            double b = floor((sample - (1.0 - p)) * (3.0 / p));
            unsigned branch = b >= 255.0 ? 255u : (unsigned)b; /* `as u8` saturates */
            const int gate = branch == 0 ? QF_GATE_X : (branch == 1 ? QF_GATE_Y : QF_GATE_Z);
            return qfo_sv_apply(amps, n, gate, 0.0, qubit, 0);
        }
        return 0;
    }
    if (channel == QF_CHANNEL_AMPLITUDE_DAMPING || channel == QF_CHANNEL_PHASE_DAMPING) {
        const double gamma = p;
        if (!valid_probability(gamma)) return QF_ERR_INVALID_PROBABILITY;
        const double norm = qfo_sv_norm_sqr(amps, n);
        if (!isfinite(norm) || norm <= DBL_EPSILON) return QF_ERR_INVALID_PROBABILITY;
        const double probability_one = p_one_sum(a, dim, mask);
        const double jump_probability = clamp01(gamma * probability_one / norm);
        const int jump = qfo_rng_next_f64(rng_state) < jump_probability;
        const double branch_norm = jump ? gamma * probability_one : norm - gamma * probability_one;
        if (!isfinite(branch_norm) || branch_norm <= DBL_EPSILON) return QF_ERR_INVALID_PROBABILITY;
        const double inverse_norm = 1.0 / sqrt(branch_norm);
        if (jump) {
            const double scale = sqrt(gamma) * inverse_norm;
            for (uint64_t base = 0; base < dim; ++base) {
                if (base & mask) continue;
                const uint64_t excited = base | mask;
                const cplx value = c_mulf(a[excited], scale);
                if (channel == QF_CHANNEL_AMPLITUDE_DAMPING) {
                    a[base] = value;
                    a[excited] = c_new(0.0, 0.0);
                } else {
                    a[base] = c_new(0.0, 0.0);
                    a[excited] = value;
                }
            }
        } else {
            const double excited_scale = sqrt(1.0 - gamma) * inverse_norm;
            for (uint64_t i = 0; i < dim; ++i) a[i] = c_mulf(a[i], (i & mask) == 0 ? inverse_norm : excited_scale);
        }
        return 0;
    }
    if (channel == QF_CHANNEL_THERMAL_DAMPING) {
        const double gamma_down = p;
        if (!valid_probability(gamma_down)) return QF_ERR_INVALID_PROBABILITY;
        if (!isfinite(beta_delta) || beta_delta < 0.0) return QF_ERR_INVALID_PROBABILITY;
        const double gamma_up = gamma_down * exp(-beta_delta);
        const double norm = qfo_sv_norm_sqr(amps, n);
        if (!isfinite(norm) || norm <= DBL_EPSILON) return QF_ERR_INVALID_PROBABILITY;
        const double probability_one = p_one_sum(a, dim, mask);
        const double p1 = clamp01(probability_one / norm);
        const double p0 = 1.0 - p1;
        const double down = p1 * gamma_down;
        const double up = p0 * gamma_up;
        const double stay = p0 * (1.0 - gamma_up) + p1 * (1.0 - gamma_down);
        const double sample = qfo_rng_next_f64(rng_state);
        double branch_norm;
        int branch;
        if (sample < down) { branch_norm = down; branch = 1; }
        else if (sample < down + up) { branch_norm = up; branch = 2; }
        else { branch_norm = stay; branch = 0; }
        if (!isfinite(branch_norm) || branch_norm <= DBL_EPSILON) return QF_ERR_INVALID_PROBABILITY;
        const double inverse_norm = 1.0 / sqrt(branch_norm);
        if (branch == 1) {
            const double scale = sqrt(gamma_down) * inverse_norm;
            for (uint64_t base = 0; base < dim; ++base) {
                if (base & mask) continue;
                a[base] = c_mulf(a[base | mask], scale);
                a[base | mask] = c_new(0.0, 0.0);
            }
        } else if (branch == 2) {
            const double scale = sqrt(gamma_up) * inverse_norm;
            for (uint64_t base = 0; base < dim; ++base) {
                if (base & mask) continue;
                a[base | mask] = c_mulf(a[base], scale);
                a[base] = c_new(0.0, 0.0);
            }
        } else {
            const double ground_scale = sqrt(1.0 - gamma_up) * inverse_norm;
            const double excited_scale = sqrt(1.0 - gamma_down) * inverse_norm;
            for (uint64_t i = 0; i < dim; ++i) a[i] = c_mulf(a[i], (i & mask) == 0 ? ground_scale : excited_scale);
        }
        return 0;
    }
    return QF_ERR_INVALID_ARGUMENT;
}

/* PauliWord::apply_basis_index (src/analytic.rs:2629-2650): P|i> = phase |i'>.
 * Qubits are visited in increasing order; phases are exact (+-1, +-i). */
static uint64_t pauli_apply_basis_index(uint64_t xmask, uint64_t zmask, uint32_t n, uint64_t index, cplx *phase) {
    cplx ph = c_new(1.0, 0.0);
    for (uint32_t q = 0; q < n; ++q) {
        uint64_t m = 1ULL << q;
        int bit_one = (index & m) != 0;
        int x = (xmask & m) != 0, z = (zmask & m) != 0;
        if (x && z) { /* Y */
            ph = c_mul(ph, bit_one ? c_new(0.0, -1.0) : c_new(0.0, 1.0));
            index ^= m;
        } else if (x) {
            index ^= m;
        } else if (z && bit_one) {
            ph = c_mulf(ph, -1.0);
        }
    }
    *phase = ph;
    return index;
}

/* <psi|H|psi> term by term: <psi|P|psi> = sum_i conj(psi_i') * phase * psi_i,
 * the matrix element that PauliSum::expectation_ket (src/analytic.rs:2775)
 * reads from its sparse operator. Summation is per term in index order (the
 * reference sums CSR rows; only the rounding order differs). */
int qfo_sv_expectation_pauli_sum(const double *amps, uint32_t n, const qf_pauli_term *terms,
                                 uint64_t n_terms, double out[2]) {
    const uint64_t dim = 1ULL << n;
    const uint64_t valid = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    cplx total = c_new(0.0, 0.0);
    for (uint64_t t = 0; t < n_terms; ++t) {
        if ((terms[t].xmask | terms[t].zmask) & ~valid) return QF_ERR_QUBIT_OUT_OF_RANGE;
        cplx acc = c_new(SUM_INIT, SUM_INIT);
        for (uint64_t i = 0; i < dim; ++i) {
            cplx ph;
            uint64_t j = pauli_apply_basis_index(terms[t].xmask, terms[t].zmask, n, i, &ph);
            acc = c_add(acc, c_mul(c_conj(AMP(amps, j)), c_mul(ph, AMP(amps, i))));
        }
        total = c_add(total, c_mul(c_new(terms[t].coeff_re, terms[t].coeff_im), acc));
    }
    out[0] = total.re;
    out[1] = total.im;
    return 0;
}

/* (P|psi>) into dst: dst[i'] += coeff * phase * psi[i]. */
static void pauli_sum_apply(const cplx *src, cplx *dst, uint32_t n, const qf_pauli_term *terms, uint64_t n_terms) {
    const uint64_t dim = 1ULL << n;
    for (uint64_t i = 0; i < dim; ++i) dst[i] = c_new(0.0, 0.0);
    for (uint64_t t = 0; t < n_terms; ++t) {
        cplx c = c_new(terms[t].coeff_re, terms[t].coeff_im);
        for (uint64_t i = 0; i < dim; ++i) {
            cplx ph;
            uint64_t j = pauli_apply_basis_index(terms[t].xmask, terms[t].zmask, n, i, &ph);
            dst[j] = c_add(dst[j], c_mul(c, c_mul(ph, src[i])));
        }
    }
}

/* ---- Circuit / ParameterizedCircuit execution --------------------------- */

/* validate_parameters / validate_inputs (src/lib.rs:4651-4675). */
static int validate_values(const double *v, uint64_t got, uint64_t expected, int count_err) {
    if (got != expected) return count_err;
    for (uint64_t k = 0; k < got; ++k)
        if (!isfinite(v[k])) return QF_ERR_NON_FINITE_PARAMETER;
    return 0;
}

/* Resolve one op to a concrete 1q gate (gate, theta); returns 1 if the op is
 * a 1q gate, 0 if it is a 2q op, <0 for an error status (negated). */
static int resolve_gate(const qf_op *op, const double *params, uint64_t n_params,
                        const double *inputs, uint64_t n_inputs, int64_t index,
                        int64_t shift_op, double shift_delta, int *gate, double *theta) {
    switch (op->kind) {
    case QF_OP_GATE:
        *gate = op->gate; *theta = op->theta;
        return 1;
    case QF_OP_ROTATION:
        if (op->param >= n_params) return -QF_ERR_INVALID_PARAMETER_COUNT;
        *gate = rotation_gate(op->gate);
        *theta = params[op->param] + (shift_op == index ? shift_delta : 0.0);
        return 1;
    case QF_OP_ENCODING:
        if (op->param >= n_inputs) return -QF_ERR_INVALID_INPUT_COUNT;
        *gate = rotation_gate(op->gate);
        *theta = inputs[op->param];
        return 1;
    default:
        return 0;
    }
}

/* Apply one non-measurement op. `shift_op`/`shift_delta` follow run_with_shift
 * (src/lib.rs:4677-4740): the delta is added to the rotation at that index. */
static int apply_op(double *amps, uint32_t n, const qf_op *op, const double *params, uint64_t n_params,
                    const double *inputs, uint64_t n_inputs, int64_t index, int64_t shift_op,
                    double shift_delta, int threads) {
    int gate; double theta;
    int r = resolve_gate(op, params, n_params, inputs, n_inputs, index, shift_op, shift_delta, &gate, &theta);
    if (r < 0) return -r;
    if (r == 1) {
        return qfo_sv_apply(amps, n, gate, theta, op->q0, threads);
    }
    switch (op->kind) {
    case QF_OP_CNOT: return qfo_sv_apply_cnot(amps, n, op->q0, op->q1);
    case QF_OP_CZ: return qfo_sv_apply_cz(amps, n, op->q0, op->q1);
    case QF_OP_SWAP: return qfo_sv_apply_swap(amps, n, op->q0, op->q1);
    case QF_OP_CHANNEL: return QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX;
    case QF_OP_MEASURE: case QF_OP_COND: return QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION;
    default: return QF_ERR_INVALID_ARGUMENT;
    }
}

/* Circuit::run (src/lib.rs:2786-2802) and ParameterizedCircuit::run_with_shift
 * (src/lib.rs:4677-4740). Parameters/inputs are validated only when the list
 * holds parameterised ops (a plain Circuit has none). */
int qfo_run_ops(double *amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                int64_t shift_op, double shift_delta, int threads) {
    int st = validate_values(inputs, n_inputs, n_inputs, QF_ERR_INVALID_INPUT_COUNT);
    if (!st) st = validate_values(params, n_params, n_params, QF_ERR_INVALID_PARAMETER_COUNT);
    if (st) return st;
    for (uint64_t k = 0; k < n_ops; ++k) {
        st = apply_op(amps, n, &ops[k], params, n_params, inputs, n_inputs, (int64_t)k, shift_op, shift_delta, threads);
        if (st) return st;
    }
    return 0;
}

/* Classical register width and validation (src/lib.rs:2853-2873). */
static int classical_width(const qf_op *ops, uint64_t n_ops, uint32_t *width) {
    uint32_t w = 0;
    for (uint64_t k = 0; k < n_ops; ++k) {
        if (ops[k].kind == QF_OP_MEASURE || ops[k].kind == QF_OP_COND) {
            if (ops[k].param >= 4096) return QF_ERR_CLASSICAL_BIT_OUT_OF_RANGE;
            if (ops[k].param + 1 > w) w = ops[k].param + 1;
        }
    }
    *width = w;
    return 0;
}

/* Circuit::run_shots_impl (src/lib.rs:2842-2916): every shot clones the
 * initial state (normalised first when allow_noise) and re-runs every op;
 * measurements and channel trajectories draw from one SmallRng in shot-major
 * order. Without allow_noise a channel is rejected as density-matrix work.
 * outcomes[s] packs classical bit c at bit c (registers wider than 64 bits
 * are rejected here). */
static int run_shots_literal(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops, uint64_t shots,
                             uint64_t seed, int allow_noise, uint64_t *outcomes, uint32_t *width) {
    if (shots == 0) return QF_ERR_INVALID_SHOT_COUNT;
    uint32_t w;
    int st = classical_width(ops, n_ops, &w);
    if (st) return st;
    if (w > 64) return QF_ERR_UNSUPPORTED_OPERATION;
    *width = w;
    const uint64_t dim = 1ULL << n;
    double *start = (double *)malloc(sizeof(double) * 2 * dim);
    double *state = (double *)malloc(sizeof(double) * 2 * dim);
    if (!start || !state) {
        free(start);
        free(state);
        return QF_ERR_MEMORY_ALLOCATION_FAILED;
    }
    memcpy(start, init_amps, sizeof(double) * 2 * dim);
    /* normalize() gives the same state in every shot: done once */
    if (allow_noise) st = qfo_sv_normalize(start, n);
    uint64_t rng = qfo_rng_seeded(seed);
    for (uint64_t s = 0; s < shots && !st; ++s) {
        memcpy(state, start, sizeof(double) * 2 * dim);
        uint64_t classical = 0;
        for (uint64_t k = 0; k < n_ops && !st; ++k) {
            const qf_op *op = &ops[k];
            if (op->kind == QF_OP_MEASURE) {
                uint8_t o;
                st = qfo_sv_measure(state, n, op->q0, &rng, &o);
                if (!st) classical = (classical & ~(1ULL << op->param)) | ((uint64_t)o << op->param);
            } else if (op->kind == QF_OP_COND) {
                if (((classical >> op->param) & 1ULL) == (uint64_t)(op->flags & 1))
                    st = qfo_sv_apply(state, n, op->gate, op->theta, op->q0, 0);
            } else if (op->kind == QF_OP_CHANNEL && allow_noise) {
                st = qfo_sv_channel_trajectory(state, n, op->gate, op->theta, qf_op_aux(op), op->q0, &rng);
            } else {
                st = apply_op(state, n, op, NULL, 0, NULL, 0, (int64_t)k, -1, 0.0, 0);
            }
        }
        outcomes[s] = classical;
    }
    free(start);
    free(state);
    return st;
}

int qfo_run_shots_literal(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                          uint64_t shots, uint64_t seed, uint64_t *outcomes, uint32_t *width) {
    return run_shots_literal(init_amps, n, ops, n_ops, shots, seed, 0, outcomes, width);
}

/* Circuit::run_shots_with_noise (src/lib.rs:2829-2840). */
int qfo_run_shots_noisy_literal(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                                uint64_t shots, uint64_t seed, uint64_t *outcomes, uint32_t *width) {
    return run_shots_literal(init_amps, n, ops, n_ops, shots, seed, 1, outcomes, width);
}

/* Memoised exact form of run_shots_impl for circuits whose measurements all
 * follow the last gate. Because the pre-measurement state is the same in
 * every shot, the state after measuring (q_0..q_{k-1}) with outcomes b is the
 * initial state restricted to the indices consistent with b and divided, in
 * order, by s_0, ..., s_{k-1}; p_one for that prefix is the reference's
 * sequential index-order sum of norm_sqr of those divided amplitudes
 * (src/lib.rs:1329-1346). The tree memoises p_one per (level, prefix), so each
 * shot costs m table look-ups and every value is bit-identical to the literal
 * per-shot re-simulation. */
typedef struct {
    double *p_one;      /* per level, 2^level entries */
    uint8_t *done;
} tree_level;

static double tree_p_one(const cplx *psi, uint32_t n, const uint32_t *mq, uint32_t k, uint64_t prefix,
                         const double *scales) {
    /* indices consistent with prefix: bit mq[j] == bit j of prefix for j < k */
    uint64_t fixed_mask = 0, fixed_val = 0;
    int conflict = 0;
    for (uint32_t j = 0; j < k; ++j) {
        uint64_t m = 1ULL << mq[j];
        uint64_t v = ((prefix >> j) & 1ULL) ? m : 0;
        if ((fixed_mask & m) && ((fixed_val & m) != v)) conflict = 1;
        fixed_mask |= m;
        fixed_val |= v;
    }
    const uint64_t qmask = 1ULL << mq[k];
    double sum = SUM_INIT;
    if (conflict) return sum; /* every consistent amplitude was zeroed */
    const uint64_t free_mask = ((n >= 64) ? ~0ULL : ((1ULL << n) - 1)) & ~fixed_mask;
    /* enumerate free bits in increasing index order */
    uint64_t sub = 0;
    for (;;) {
        uint64_t i = fixed_val | sub;
        if (i & qmask) {
            cplx a = psi[i];
            for (uint32_t j = 0; j < k; ++j) a = c_divf(a, scales[j]);
            sum += c_norm_sqr(a);
        }
        if (sub == free_mask) break;
        sub = (sub - free_mask) & free_mask;
    }
    return sum;
}

int qfo_run_shots_tree(const double *init_amps, uint32_t n, const qf_op *ops, uint64_t n_ops,
                       uint64_t shots, uint64_t seed, uint64_t *outcomes, uint32_t *width, int threads) {
    if (shots == 0) return QF_ERR_INVALID_SHOT_COUNT;
    uint32_t w;
    int st = classical_width(ops, n_ops, &w);
    if (st) return st;
    if (w > 64) return QF_ERR_UNSUPPORTED_OPERATION;
    *width = w;
    /* split into unitary prefix + terminal measurements */
    uint64_t first_measure = n_ops;
    for (uint64_t k = 0; k < n_ops; ++k)
        if (ops[k].kind == QF_OP_MEASURE) { first_measure = k; break; }
    uint32_t m = 0;
    for (uint64_t k = first_measure; k < n_ops; ++k) {
        if (ops[k].kind != QF_OP_MEASURE) return QF_ERR_UNSUPPORTED_OPERATION;
        if (ops[k].q0 >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
        ++m;
    }
    for (uint64_t k = 0; k < first_measure; ++k)
        if (ops[k].kind == QF_OP_COND) return QF_ERR_UNSUPPORTED_OPERATION;
    if (m > 30) return QF_ERR_UNSUPPORTED_OPERATION;
    const uint64_t dim = 1ULL << n;
    double *psi = (double *)malloc(sizeof(double) * 2 * dim);
    if (!psi) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    memcpy(psi, init_amps, sizeof(double) * 2 * dim);
    st = qfo_run_ops(psi, n, ops, first_measure, NULL, 0, NULL, 0, -1, 0.0, threads);
    uint32_t *mq = (uint32_t *)malloc(sizeof(uint32_t) * (m + 1));
    uint32_t *mc = (uint32_t *)malloc(sizeof(uint32_t) * (m + 1));
    tree_level *lv = (tree_level *)calloc(m + 1, sizeof(tree_level));
    for (uint32_t j = 0; j < m; ++j) {
        mq[j] = ops[first_measure + j].q0;
        mc[j] = ops[first_measure + j].param;
        lv[j].p_one = (double *)malloc(sizeof(double) * (1ULL << j));
        lv[j].done = (uint8_t *)calloc(1ULL << j, 1);
        if (!lv[j].p_one || !lv[j].done) st = QF_ERR_MEMORY_ALLOCATION_FAILED;
    }
    double scales[64];
    uint64_t rng = qfo_rng_seeded(seed);
    for (uint64_t s = 0; s < shots && !st; ++s) {
        uint64_t prefix = 0, classical = 0;
        for (uint32_t k = 0; k < m && !st; ++k) {
            if (!lv[k].done[prefix]) {
                double p = tree_p_one((const cplx *)psi, n, mq, k, prefix, scales);
                lv[k].p_one[prefix] = p;
                lv[k].done[prefix] = 1;
            }
            double p_one = lv[k].p_one[prefix];
            if (p_one < 0.0) p_one = 0.0;
            if (p_one > 1.0) p_one = 1.0;
            uint8_t o = qfo_rng_next_f64(&rng) < p_one ? 1 : 0;
            double probability = o == 1 ? p_one : 1.0 - p_one;
            if (probability <= DBL_EPSILON) { st = QF_ERR_INVALID_PROBABILITY; break; }
            scales[k] = sqrt(probability);
            prefix |= (uint64_t)o << k;
            classical = (classical & ~(1ULL << mc[k])) | ((uint64_t)o << mc[k]);
        }
        outcomes[s] = classical;
    }
    for (uint32_t j = 0; j < m; ++j) { free(lv[j].p_one); free(lv[j].done); }
    free(lv); free(mq); free(mc); free(psi);
    return st;
}

/* ---- Gradients ----------------------------------------------------------- */

static int check_terms(uint32_t n, const qf_pauli_term *terms, uint64_t n_terms) {
    const uint64_t valid = n >= 64 ? ~0ULL : ((1ULL << n) - 1);
    for (uint64_t t = 0; t < n_terms; ++t)
        if ((terms[t].xmask | terms[t].zmask) & ~valid) return QF_ERR_QUBIT_OUT_OF_RANGE;
    return 0;
}

static int expectation_of(const double *amps, uint32_t n, const qf_pauli_term *terms, uint64_t n_terms, double *e) {
    double out[2];
    int st = qfo_sv_expectation_pauli_sum(amps, n, terms, n_terms, out);
    *e = out[0];
    return st;
}

/* One-qubit Pauli observables go through StateVector::expectation exactly as
 * the reference does (src/lib.rs:3536-3543); longer sums term by term. */
static int observable_value(const double *amps, uint32_t n, const qf_pauli_term *terms, uint64_t n_terms, double *e) {
    if (n_terms == 1 && terms[0].coeff_re == 1.0 && terms[0].coeff_im == 0.0) {
        uint64_t x = terms[0].xmask, z = terms[0].zmask, u = x | z;
        if (u && !(u & (u - 1))) {
            uint32_t q = 0;
            while (!((u >> q) & 1ULL)) ++q;
            int obs = (x && z) ? QF_PAULI_Y : x ? QF_PAULI_X : QF_PAULI_Z;
            return qfo_sv_expectation(amps, n, obs, q, e);
        }
    }
    return expectation_of(amps, n, terms, n_terms, e);
}

int qfo_expectation(uint32_t n, const qf_op *ops, uint64_t n_ops,
                    const double *params, uint64_t n_params, const double *inputs, uint64_t n_inputs,
                    const qf_pauli_term *terms, uint64_t n_terms, double *energy, int threads) {
    if (n == 0) return QF_ERR_ZERO_QUBITS;
    int st = check_terms(n, terms, n_terms);
    if (st) return st;
    double *psi = (double *)malloc(sizeof(double) * 2 * (1ULL << n));
    if (!psi) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    qfo_sv_zero(psi, n);
    st = qfo_run_ops(psi, n, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, threads);
    if (!st) st = observable_value(psi, n, terms, n_terms, energy);
    free(psi);
    return st;
}

/* parameter_shift_gradient_with_inputs (src/lib.rs:3516-3546): for every
 * rotation occurrence, g[p] += 0.5 * (E(+pi/2) - E(-pi/2)). */
int qfo_parameter_shift_gradient(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                 const double *params, uint64_t n_params,
                                 const double *inputs, uint64_t n_inputs,
                                 const qf_pauli_term *terms, uint64_t n_terms, double *grad, int threads) {
    if (n == 0) return QF_ERR_ZERO_QUBITS;
    int st = validate_values(inputs, n_inputs, n_inputs, QF_ERR_INVALID_INPUT_COUNT);
    if (!st) st = validate_values(params, n_params, n_params, QF_ERR_INVALID_PARAMETER_COUNT);
    if (!st) st = check_terms(n, terms, n_terms);
    if (st) return st;
    const double shift = 1.57079632679489661923; /* FRAC_PI_2 */
    for (uint64_t p = 0; p < n_params; ++p) grad[p] = 0.0;
    double *psi = (double *)malloc(sizeof(double) * 2 * (1ULL << n));
    if (!psi) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    for (uint64_t k = 0; k < n_ops && !st; ++k) {
        if (ops[k].kind != QF_OP_ROTATION) continue;
        double plus, minus;
        qfo_sv_zero(psi, n);
        st = qfo_run_ops(psi, n, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, shift, threads);
        if (!st) st = observable_value(psi, n, terms, n_terms, &plus);
        if (st) break;
        qfo_sv_zero(psi, n);
        st = qfo_run_ops(psi, n, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, -shift, threads);
        if (!st) st = observable_value(psi, n, terms, n_terms, &minus);
        if (st) break;
        grad[ops[k].param] += 0.5 * (plus - minus);
    }
    free(psi);
    return st;
}

/* finite_difference_gradient_with_inputs (src/gradients.rs:344-375). */
int qfo_finite_difference_gradient(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                   const double *params, uint64_t n_params,
                                   const double *inputs, uint64_t n_inputs,
                                   const qf_pauli_term *terms, uint64_t n_terms, double step,
                                   double *grad, int threads) {
    if (!isfinite(step) || step <= 0.0) return QF_ERR_INVALID_FINITE_DIFFERENCE_STEP;
    if (n == 0) return QF_ERR_ZERO_QUBITS;
    int st = validate_values(inputs, n_inputs, n_inputs, QF_ERR_INVALID_INPUT_COUNT);
    if (!st) st = validate_values(params, n_params, n_params, QF_ERR_INVALID_PARAMETER_COUNT);
    if (!st) st = check_terms(n, terms, n_terms);
    if (st) return st;
    for (uint64_t p = 0; p < n_params; ++p) grad[p] = 0.0;
    double *psi = (double *)malloc(sizeof(double) * 2 * (1ULL << n));
    if (!psi) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    for (uint64_t k = 0; k < n_ops && !st; ++k) {
        if (ops[k].kind != QF_OP_ROTATION) continue;
        double plus, minus;
        qfo_sv_zero(psi, n);
        st = qfo_run_ops(psi, n, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, step, threads);
        if (!st) st = observable_value(psi, n, terms, n_terms, &plus);
        if (st) break;
        qfo_sv_zero(psi, n);
        st = qfo_run_ops(psi, n, ops, n_ops, params, n_params, inputs, n_inputs, (int64_t)k, -step, threads);
        if (!st) st = observable_value(psi, n, terms, n_terms, &minus);
        if (st) break;
        grad[ops[k].param] += (plus - minus) / (2.0 * step);
    }
    free(psi);
    return st;
}

/* The Pauli generator of a rotation axis (src/gradients.rs:509-515). */
static int generator_gate(int axis) {
    return axis == QF_PAULI_X ? QF_GATE_X : axis == QF_PAULI_Y ? QF_GATE_Y : QF_GATE_Z;
}

/* 2 * sum Re(conj(lambda_i) * ((P psi)_i * (-i/2))) in index order
 * (src/lib.rs:3648-3664). `scratch` receives P|psi>. */
static double overlap_term(const cplx *lambda, const cplx *after, cplx *scratch, uint32_t n, int axis, uint32_t target) {
    const uint64_t dim = 1ULL << n;
    memcpy(scratch, after, sizeof(cplx) * dim);
    qfo_sv_apply((double *)scratch, n, generator_gate(axis), 0.0, target, 0);
    const cplx minus_i_half = c_new(0.0, -0.5);
    double s = SUM_INIT;
    for (uint64_t i = 0; i < dim; ++i) s += c_mul(c_conj(lambda[i]), c_mul(scratch[i], minus_i_half)).re;
    return 2.0 * s;
}

/* Inverse of op k applied to v (the costate propagation of
 * src/lib.rs:3672-3700): adjoint_gate for fixed gates, -theta for rotations,
 * self-inverse 2q gates. */
static int apply_inverse(double *v, uint32_t n, const qf_op *op, const double *params, const double *inputs) {
    switch (op->kind) {
    case QF_OP_GATE: {
        int g; double t;
        adjoint_gate(op->gate, op->theta, &g, &t);
        return qfo_sv_apply(v, n, g, t, op->q0, 0);
    }
    case QF_OP_ROTATION: return qfo_sv_apply(v, n, rotation_gate(op->gate), -params[op->param], op->q0, 0);
    case QF_OP_ENCODING: return qfo_sv_apply(v, n, rotation_gate(op->gate), -inputs[op->param], op->q0, 0);
    case QF_OP_CNOT: return qfo_sv_apply_cnot(v, n, op->q0, op->q1);
    case QF_OP_CZ: return qfo_sv_apply_cz(v, n, op->q0, op->q1);
    case QF_OP_SWAP: return qfo_sv_apply_swap(v, n, op->q0, op->q1);
    case QF_OP_CHANNEL: return QF_ERR_OPERATION_REQUIRES_DENSITY_MATRIX;
    default: return QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION;
    }
}

/* Costate lambda = H|psi>. For one unit-coefficient Pauli on one qubit this is
 * the reference's `costate.apply(pauli, observable_qubit)` (src/lib.rs:3623-3632). */
static void make_costate(const cplx *psi, cplx *lambda, uint32_t n, const qf_pauli_term *terms, uint64_t n_terms) {
    const uint64_t dim = 1ULL << n;
    if (n_terms == 1 && terms[0].coeff_re == 1.0 && terms[0].coeff_im == 0.0) {
        uint64_t x = terms[0].xmask, z = terms[0].zmask, u = x | z;
        if (u && !(u & (u - 1))) {
            uint32_t q = 0;
            while (!((u >> q) & 1ULL)) ++q;
            int g = (x && z) ? QF_GATE_Y : x ? QF_GATE_X : QF_GATE_Z;
            memcpy(lambda, psi, sizeof(cplx) * dim);
            qfo_sv_apply((double *)lambda, n, g, 0.0, q, 0);
            return;
        }
    }
    pauli_sum_apply(psi, lambda, n, terms, n_terms);
}

/* adjoint_gradient_with_inputs (src/lib.rs:3564-3704): forward sweep storing
 * every intermediate state, costate = O psi, reverse sweep accumulating
 * 2 Re <lambda|(-i/2) P psi_after> and propagating lambda <- U^dagger lambda.
 * backprop_gradient_with_inputs (src/gradients.rs:392-506) is the same
 * computation. The observable may be a Pauli sum (the reference takes one
 * single-qubit Pauli). O(ops * 2^n) memory: small n only. */
int qfo_adjoint_gradient_stored(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                const double *params, uint64_t n_params,
                                const double *inputs, uint64_t n_inputs,
                                const qf_pauli_term *terms, uint64_t n_terms, double *grad) {
    if (n == 0) return QF_ERR_ZERO_QUBITS;
    int st = validate_values(inputs, n_inputs, n_inputs, QF_ERR_INVALID_INPUT_COUNT);
    if (!st) st = validate_values(params, n_params, n_params, QF_ERR_INVALID_PARAMETER_COUNT);
    if (!st) st = check_terms(n, terms, n_terms);
    if (st) return st;
    const uint64_t dim = 1ULL << n;
    cplx *states = (cplx *)malloc(sizeof(cplx) * dim * (n_ops + 1));
    cplx *lambda = (cplx *)malloc(sizeof(cplx) * dim);
    cplx *scratch = (cplx *)malloc(sizeof(cplx) * dim);
    if (!states || !lambda || !scratch) { free(states); free(lambda); free(scratch); return QF_ERR_MEMORY_ALLOCATION_FAILED; }
    qfo_sv_zero((double *)states, n);
    for (uint64_t k = 0; k < n_ops && !st; ++k) {
        memcpy(states + dim * (k + 1), states + dim * k, sizeof(cplx) * dim);
        st = apply_op((double *)(states + dim * (k + 1)), n, &ops[k], params, n_params, inputs, n_inputs,
                      (int64_t)k, -1, 0.0, 0);
    }
    if (!st) {
        for (uint64_t p = 0; p < n_params; ++p) grad[p] = 0.0;
        make_costate(states + dim * n_ops, lambda, n, terms, n_terms);
        for (uint64_t kk = n_ops; kk-- > 0 && !st;) {
            const qf_op *op = &ops[kk];
            if (op->kind == QF_OP_ROTATION)
                grad[op->param] += overlap_term(lambda, states + dim * (kk + 1), scratch, n, op->gate, op->q0);
            st = apply_inverse((double *)lambda, n, op, params, inputs);
        }
    }
    free(states); free(lambda); free(scratch);
    return st;
}

/* The same gradient with O(2^n) memory: psi is uncomputed gate by gate
 * instead of stored. Also returns <H>. Used as the oracle at sizes where the
 * stored form does not fit. */
int qfo_adjoint_gradient_uncompute(uint32_t n, const qf_op *ops, uint64_t n_ops,
                                   const double *params, uint64_t n_params,
                                   const double *inputs, uint64_t n_inputs,
                                   const qf_pauli_term *terms, uint64_t n_terms,
                                   double *energy, double *grad, int threads) {
    if (n == 0) return QF_ERR_ZERO_QUBITS;
    int st = validate_values(inputs, n_inputs, n_inputs, QF_ERR_INVALID_INPUT_COUNT);
    if (!st) st = validate_values(params, n_params, n_params, QF_ERR_INVALID_PARAMETER_COUNT);
    if (!st) st = check_terms(n, terms, n_terms);
    if (st) return st;
    const uint64_t dim = 1ULL << n;
    cplx *psi = (cplx *)malloc(sizeof(cplx) * dim);
    cplx *lambda = (cplx *)malloc(sizeof(cplx) * dim);
    cplx *scratch = (cplx *)malloc(sizeof(cplx) * dim);
    if (!psi || !lambda || !scratch) { free(psi); free(lambda); free(scratch); return QF_ERR_MEMORY_ALLOCATION_FAILED; }
    qfo_sv_zero((double *)psi, n);
    st = qfo_run_ops((double *)psi, n, ops, n_ops, params, n_params, inputs, n_inputs, -1, 0.0, threads);
    if (!st && energy) st = observable_value((double *)psi, n, terms, n_terms, energy);
    if (!st) {
        for (uint64_t p = 0; p < n_params; ++p) grad[p] = 0.0;
        make_costate(psi, lambda, n, terms, n_terms);
        for (uint64_t kk = n_ops; kk-- > 0 && !st;) {
            const qf_op *op = &ops[kk];
            if (op->kind == QF_OP_ROTATION)
                grad[op->param] += overlap_term(lambda, psi, scratch, n, op->gate, op->q0);
            st = apply_inverse((double *)psi, n, op, params, inputs);
            if (!st) st = apply_inverse((double *)lambda, n, op, params, inputs);
        }
    }
    free(psi); free(lambda); free(scratch);
    return st;
}

/* ---- MaxCut (src/qaoa_transfer.rs:199-218, src/mps_qaoa.rs:58-95) ------- */
double qfo_maxcut_expectation(const double *amps, uint32_t n, const uint32_t *edges_uv,
                              const double *weights, uint64_t n_edges) {
    const uint64_t dim = 1ULL << n;
    double total = 0.0;
    for (uint64_t i = 0; i < dim; ++i) {
        double probability = c_norm_sqr(AMP(amps, i));
        if (probability == 0.0) continue;
        double cut = 0.0;
        for (uint64_t e = 0; e < n_edges; ++e)
            if (((i >> edges_uv[2 * e]) ^ (i >> edges_uv[2 * e + 1])) & 1ULL) cut += weights[e];
        total += probability * cut;
    }
    return total;
}

/* MaxCutProblem::random_3_regular: configuration model, seeded Fisher-Yates,
 * retry on self-loops and multi-edges, edges sorted by (u, v). Writes 3n/2
 * (u, v) pairs. */
int qfo_random_3_regular(uint32_t n, uint64_t seed, uint32_t *edges_uv) {
    if (n < 4 || (n % 2) != 0) return QF_ERR_INVALID_ARGUMENT;
    uint64_t rng = qfo_rng_seeded(seed);
    const uint32_t ns = 3 * n, ne = ns / 2;
    uint32_t *stubs = (uint32_t *)malloc(sizeof(uint32_t) * ns);
    uint32_t *eu = (uint32_t *)malloc(sizeof(uint32_t) * ne * 2);
    if (!stubs || !eu) { free(stubs); free(eu); return QF_ERR_MEMORY_ALLOCATION_FAILED; }
    int found = 0;
    for (int attempt = 0; attempt < 10000 && !found; ++attempt) {
        for (uint32_t v = 0; v < n; ++v) stubs[3 * v] = stubs[3 * v + 1] = stubs[3 * v + 2] = v;
        for (uint32_t i = ns - 1; i >= 1; --i) {
            uint32_t j = (uint32_t)(qfo_rng_next_u64(&rng) % ((uint64_t)i + 1));
            uint32_t t = stubs[i]; stubs[i] = stubs[j]; stubs[j] = t;
        }
        uint32_t count = 0;
        int ok = 1;
        for (uint32_t p = 0; p < ne && ok; ++p) {
            uint32_t a = stubs[2 * p], b = stubs[2 * p + 1];
            if (a == b) { ok = 0; break; }
            uint32_t u = a < b ? a : b, v = a < b ? b : a;
            for (uint32_t e = 0; e < count; ++e)
                if (eu[2 * e] == u && eu[2 * e + 1] == v) { ok = 0; break; }
            if (!ok) break;
            eu[2 * count] = u; eu[2 * count + 1] = v; ++count;
        }
        if (ok) found = 1;
    }
    if (found) {
        /* sort_by_key((u, v)) — stable insertion sort on distinct keys */
        for (uint32_t i = 1; i < ne; ++i) {
            uint32_t u = eu[2 * i], v = eu[2 * i + 1];
            int64_t j = (int64_t)i - 1;
            while (j >= 0 && (eu[2 * j] > u || (eu[2 * j] == u && eu[2 * j + 1] > v))) {
                eu[2 * (j + 1)] = eu[2 * j]; eu[2 * (j + 1) + 1] = eu[2 * j + 1]; --j;
            }
            eu[2 * (j + 1)] = u; eu[2 * (j + 1) + 1] = v;
        }
        memcpy(edges_uv, eu, sizeof(uint32_t) * ne * 2);
    }
    free(stubs); free(eu);
    return found ? 0 : QF_ERR_UNSUPPORTED_OPERATION;
}

/* ---- DensityMatrix (src/lib.rs:1551-2235) -------------------------------
 * Row-major entries rho[row * D + col], D = 2^n, interleaved f64. */

/* DensityMatrix::from_state (src/lib.rs:1641-1655): rho = |psi><psi|. */
void qfo_dm_from_state(const double *amps, uint32_t n, double *rho) {
    const uint64_t D = 1ULL << n;
    const cplx *a = (const cplx *)amps;
    cplx *r = (cplx *)rho;
    for (uint64_t row = 0; row < D; ++row)
        for (uint64_t col = 0; col < D; ++col) r[row * D + col] = c_mul(a[row], c_conj(a[col]));
}

/* DensityMatrix::maximally_mixed_with_memory_budget (src/lib.rs:1668-1700): I / 2^n. */
void qfo_dm_maximally_mixed(uint32_t n, double *rho) {
    const uint64_t D = 1ULL << n;
    cplx *r = (cplx *)rho;
    const double v = 1.0 / (double)D;
    for (uint64_t i = 0; i < D * D; ++i) r[i] = c_new(0.0, 0.0);
    for (uint64_t i = 0; i < D; ++i) r[i * D + i] = c_new(v, 0.0);
}

/* DensityMatrix::local_transform (src/lib.rs:2169-2206): M rho M^dagger as
 * a left pass over rows then a right pass over columns, into `out`. */
static int dm_local_transform(const cplx *e, uint64_t D, const cplx m[4], uint32_t q, cplx *out) {
    const uint64_t mask = 1ULL << q;
    cplx *left = (cplx *)malloc(sizeof(cplx) * D * D);
    if (!left) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    for (uint64_t row = 0; row < D; ++row) {
        const uint64_t row0 = row & ~mask, row1 = row0 | mask;
        for (uint64_t col = 0; col < D; ++col) {
            const cplx a = e[row0 * D + col], b = e[row1 * D + col];
            left[row * D + col] = (row & mask) == 0 ? c_add(c_mul(m[0], a), c_mul(m[1], b))
                                                    : c_add(c_mul(m[2], a), c_mul(m[3], b));
        }
    }
    for (uint64_t row = 0; row < D; ++row) {
        for (uint64_t col = 0; col < D; ++col) {
            const uint64_t col0 = col & ~mask, col1 = col0 | mask;
            const cplx a = left[row * D + col0], b = left[row * D + col1];
            out[row * D + col] = (col & mask) == 0 ? c_add(c_mul(a, c_conj(m[0])), c_mul(b, c_conj(m[1])))
                                                   : c_add(c_mul(a, c_conj(m[2])), c_mul(b, c_conj(m[3])));
        }
    }
    free(left);
    return 0;
}

/* DensityMatrix::apply (src/lib.rs:2043-2054). */
int qfo_dm_apply(double *rho, uint32_t n, int gate, double theta, uint32_t q) {
    if (q >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    cplx m[4];
    int st = gate_matrix(gate, theta, m);
    if (st) return st;
    const uint64_t D = 1ULL << n;
    cplx *out = (cplx *)malloc(sizeof(cplx) * D * D);
    if (!out) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    st = dm_local_transform((cplx *)rho, D, m, q, out);
    if (!st) memcpy(rho, out, sizeof(cplx) * D * D);
    free(out);
    return st;
}

/* DensityMatrix::apply_basis_permutation (src/lib.rs:2033-2041) for CNOT,
 * SWAP (src/lib.rs:1983-1997, 2018-2031); CZ flips signs (src/lib.rs:1999-2016). */
int qfo_dm_apply_2q(double *rho, uint32_t n, int kind, uint32_t a, uint32_t b) {
    int st = check_pair(n, a, b);
    if (st) return st;
    const uint64_t D = 1ULL << n, am = 1ULL << a, bm = 1ULL << b;
    cplx *e = (cplx *)rho;
    if (kind == QF_OP_CZ) {
        for (uint64_t row = 0; row < D; ++row)
            for (uint64_t col = 0; col < D; ++col) {
                if ((row & am) && (row & bm)) e[row * D + col] = c_mulf(e[row * D + col], -1.0);
                if ((col & am) && (col & bm)) e[row * D + col] = c_mulf(e[row * D + col], -1.0);
            }
        return 0;
    }
    cplx *orig = (cplx *)malloc(sizeof(cplx) * D * D);
    if (!orig) return QF_ERR_MEMORY_ALLOCATION_FAILED;
    memcpy(orig, e, sizeof(cplx) * D * D);
    for (uint64_t row = 0; row < D; ++row) {
        for (uint64_t col = 0; col < D; ++col) {
            uint64_t pr = row, pc = col;
            if (kind == QF_OP_CNOT) {
                if (row & am) pr ^= bm;
                if (col & am) pc ^= bm;
            } else {
                if (((row & am) == 0) != ((row & bm) == 0)) pr ^= am ^ bm;
                if (((col & am) == 0) != ((col & bm) == 0)) pc ^= am ^ bm;
            }
            e[row * D + col] = orig[pr * D + pc];
        }
    }
    free(orig);
    return 0;
}

/* apply_kraus (src/lib.rs:2145-2156): the sum of local_transform(K) in order. */
static int dm_apply_kraus(double *rho, uint32_t n, const cplx (*ops)[4], int count, uint32_t q) {
    const uint64_t D = 1ULL << n, E = D * D;
    cplx *sum = (cplx *)calloc(E, sizeof(cplx));
    cplx *branch = (cplx *)malloc(sizeof(cplx) * E);
    int st = 0;
    if (!sum || !branch) st = QF_ERR_MEMORY_ALLOCATION_FAILED;
    for (uint64_t i = 0; i < E && !st; ++i) sum[i] = c_new(0.0, 0.0);
    for (int k = 0; k < count && !st; ++k) {
        st = dm_local_transform((cplx *)rho, D, ops[k], q, branch);
        for (uint64_t i = 0; i < E && !st; ++i) sum[i] = c_add(sum[i], branch[i]);
    }
    if (!st) memcpy(rho, sum, sizeof(cplx) * E);
    free(sum);
    free(branch);
    return st;
}

/* DensityMatrix::depolarize (src/lib.rs:2208-2233). */
static int dm_depolarize(double *rho, uint32_t n, uint32_t q, double p) {
    const uint64_t D = 1ULL << n, E = D * D;
    cplx *mixed = (cplx *)malloc(sizeof(cplx) * E);
    cplx *branch = (cplx *)malloc(sizeof(cplx) * E);
    int st = 0;
    if (!mixed || !branch) st = QF_ERR_MEMORY_ALLOCATION_FAILED;
    for (uint64_t i = 0; i < E && !st; ++i) mixed[i] = c_new(0.0, 0.0);
    const int gates[3] = {QF_GATE_X, QF_GATE_Y, QF_GATE_Z};
    for (int g = 0; g < 3 && !st; ++g) {
        memcpy(branch, rho, sizeof(cplx) * E);
        st = qfo_dm_apply((double *)branch, n, gates[g], 0.0, q);
        for (uint64_t i = 0; i < E && !st; ++i) mixed[i] = c_add(mixed[i], c_mulf(branch[i], p / 3.0));
    }
    const cplx *orig = (const cplx *)rho;
    for (uint64_t i = 0; i < E && !st; ++i) mixed[i] = c_add(mixed[i], c_mulf(orig[i], 1.0 - p));
    if (!st) memcpy(rho, mixed, sizeof(cplx) * E);
    free(mixed);
    free(branch);
    return st;
}

/* DensityMatrix::apply_channel (src/lib.rs:2056-2143). */
int qfo_dm_apply_channel(double *rho, uint32_t n, int channel, double p, double beta_delta, uint32_t q) {
    if (q >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    const cplx z = c_new(0.0, 0.0), one = c_new(1.0, 0.0);
    if (channel == QF_CHANNEL_DEPOLARIZING) {
        if (!valid_probability(p)) return QF_ERR_INVALID_PROBABILITY;
        return dm_depolarize(rho, n, q, p);
    }
    if (channel == QF_CHANNEL_AMPLITUDE_DAMPING || channel == QF_CHANNEL_PHASE_DAMPING) {
        if (!valid_probability(p)) return QF_ERR_INVALID_PROBABILITY;
        cplx k[2][4] = {{one, z, z, c_new(sqrt(1.0 - p), 0.0)}, {z, z, z, z}};
        if (channel == QF_CHANNEL_AMPLITUDE_DAMPING) k[1][1] = c_new(sqrt(p), 0.0);
        else k[1][3] = c_new(sqrt(p), 0.0);
        return dm_apply_kraus(rho, n, (const cplx (*)[4])k, 2, q);
    }
    if (channel == QF_CHANNEL_THERMAL_DAMPING) {
        if (!valid_probability(p)) return QF_ERR_INVALID_PROBABILITY;
        if (!isfinite(beta_delta) || beta_delta < 0.0) return QF_ERR_INVALID_PROBABILITY;
        const double gu = p * exp(-beta_delta), gd = p;
        cplx k[3][4] = {{c_new(sqrt(1.0 - gu), 0.0), z, z, c_new(sqrt(1.0 - gd), 0.0)},
                        {z, c_new(sqrt(gd), 0.0), z, z},
                        {z, z, c_new(sqrt(gu), 0.0), z}};
        return dm_apply_kraus(rho, n, (const cplx (*)[4])k, 3, q);
    }
    return QF_ERR_INVALID_ARGUMENT;
}

/* trace (src/lib.rs:1732-1736), purity (:1738-1741). */
void qfo_dm_trace(const double *rho, uint32_t n, double out[2]) {
    const uint64_t D = 1ULL << n;
    const cplx *e = (const cplx *)rho;
    cplx t = c_new(0.0, 0.0);
    for (uint64_t i = 0; i < D; ++i) t = c_add(t, e[i * D + i]);
    out[0] = t.re;
    out[1] = t.im;
}

double qfo_dm_purity(const double *rho, uint32_t n) {
    const uint64_t E = (1ULL << n) << n;
    const cplx *e = (const cplx *)rho;
    double s = SUM_INIT;
    for (uint64_t i = 0; i < E; ++i) s += c_norm_sqr(e[i]);
    return s;
}

/* expectation_z / expectation (src/lib.rs:1858-1904), probability_one (:1906-1920). */
int qfo_dm_expectation(const double *rho, uint32_t n, int observable, uint32_t q, double *out) {
    if (q >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    const uint64_t D = 1ULL << n, mask = 1ULL << q;
    const cplx *e = (const cplx *)rho;
    if (observable == QF_PAULI_Z) {
        double s = SUM_INIT;
        for (uint64_t i = 0; i < D; ++i) s += ((i & mask) == 0 ? 1.0 : -1.0) * e[i * D + i].re;
        *out = s;
        return 0;
    }
    if (observable != QF_PAULI_X && observable != QF_PAULI_Y) return QF_ERR_INVALID_ARGUMENT;
    double v = 0.0;
    for (uint64_t row = 0; row < D; ++row) {
        if (row & mask) continue;
        const cplx c = e[row * D + (row | mask)];
        v += observable == QF_PAULI_X ? 2.0 * c.re : -2.0 * c.im;
    }
    *out = v;
    return 0;
}

int qfo_dm_probability_one(const double *rho, uint32_t n, uint32_t q, double *out) {
    if (q >= n) return QF_ERR_QUBIT_OUT_OF_RANGE;
    const uint64_t D = 1ULL << n, mask = 1ULL << q;
    const cplx *e = (const cplx *)rho;
    double s = SUM_INIT;
    for (uint64_t i = 0; i < D; ++i)
        if (i & mask) s += e[i * D + i].re;
    *out = clamp01(s);
    return 0;
}

/* DensityMatrix::measure (src/lib.rs:1922-1947). */
int qfo_dm_measure(double *rho, uint32_t n, uint32_t q, uint64_t *rng_state, uint8_t *outcome) {
    double p_one;
    int st = qfo_dm_probability_one(rho, n, q, &p_one);
    if (st) return st;
    const uint8_t o = qfo_rng_next_f64(rng_state) < p_one ? 1 : 0;
    const double probability = o == 1 ? p_one : 1.0 - p_one;
    if (probability <= DBL_EPSILON) return QF_ERR_INVALID_PROBABILITY;
    const uint64_t D = 1ULL << n, mask = 1ULL << q;
    cplx *e = (cplx *)rho;
    for (uint64_t row = 0; row < D; ++row)
        for (uint64_t col = 0; col < D; ++col) {
            if ((uint8_t)((row & mask) != 0) != o || (uint8_t)((col & mask) != 0) != o) e[row * D + col] = c_new(0.0, 0.0);
            else e[row * D + col] = c_divf(e[row * D + col], probability);
        }
    *outcome = o;
    return 0;
}

/* Circuit::run_density (src/lib.rs:2804-2818). */
int qfo_run_density(double *rho, uint32_t n, const qf_op *ops, uint64_t n_ops) {
    for (uint64_t k = 0; k < n_ops; ++k) {
        const qf_op *op = &ops[k];
        int st;
        switch (op->kind) {
        case QF_OP_GATE: st = qfo_dm_apply(rho, n, op->gate, op->theta, op->q0); break;
        case QF_OP_CNOT: case QF_OP_CZ: case QF_OP_SWAP: st = qfo_dm_apply_2q(rho, n, op->kind, op->q0, op->q1); break;
        case QF_OP_CHANNEL: st = qfo_dm_apply_channel(rho, n, op->gate, op->theta, qf_op_aux(op), op->q0); break;
        case QF_OP_MEASURE: case QF_OP_COND: st = QF_ERR_OPERATION_REQUIRES_SHOT_EXECUTION; break;
        default: st = QF_ERR_INVALID_ARGUMENT; break;
        }
        if (st) return st;
    }
    return 0;
}

/* estimate_observable_shots (src/lib.rs:4806-4838): rotate the measured basis
 * (X: H; Y: Rz(-pi/2) then H), then `shots` measurements of `qubit` on clones
 * of the state with one shared SmallRng; *successes counts outcome 0. */
int qfo_estimate_observable_shots(const double *amps, uint32_t n, int observable, uint32_t qubit, uint64_t shots,
                                  uint64_t seed, uint64_t *successes) {
    if (shots == 0) return QF_ERR_INVALID_SHOT_COUNT;
    const uint64_t dim = 1ULL << n;
    double *state = (double *)malloc(sizeof(double) * 2 * dim);
    double *sample = (double *)malloc(sizeof(double) * 2 * dim);
    int st = (!state || !sample) ? QF_ERR_MEMORY_ALLOCATION_FAILED : 0;
    if (!st) memcpy(state, amps, sizeof(double) * 2 * dim);
    if (!st && observable == QF_PAULI_X) st = qfo_sv_apply(state, n, QF_GATE_H, 0.0, qubit, 0);
    if (!st && observable == QF_PAULI_Y) {
        st = qfo_sv_apply(state, n, QF_GATE_RZ, -1.5707963267948966, qubit, 0);
        if (!st) st = qfo_sv_apply(state, n, QF_GATE_H, 0.0, qubit, 0);
    }
    uint64_t rng = qfo_rng_seeded(seed), ok = 0;
    for (uint64_t s = 0; s < shots && !st; ++s) {
        memcpy(sample, state, sizeof(double) * 2 * dim);
        uint8_t o;
        st = qfo_sv_measure(sample, n, qubit, &rng, &o);
        if (!st && o == 0) ++ok;
    }
    free(state);
    free(sample);
    if (!st) *successes = ok;
    return st;
}
