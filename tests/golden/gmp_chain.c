/*
 * Independent big-integer leg for the golden vectors: the Lucas-Lehmer / PRP
 * squaring chain computed with GMP (libgmp.so.10, called through hand-declared
 * prototypes because the image ships the library without its header).
 *
 *   PRP (mersenne2_gpu.cpp:3908, 4780): x0 = 3, x <- x^2 mod M_p, p steps,
 *        probable prime iff the final x == 9 (mersenne2_gpu.cpp:3072-3076).
 *   LL  (mersenne2_gpu.cpp:3908, 4780, 3006-3024): x0 = 4, x <- x^2 - 2 mod M_p,
 *        p-2 steps, prime iff the final x == 0 (or M_p).
 *   PRP3 (gf61 prototype .cpp:508-531): x0 = 3, x <- 3 x^2 mod M_p, p-1 steps,
 *        probable prime iff the final x == 3.
 *
 * Output: one line per checkpoint, "iter <k> res64 <16 hex>", plus, with
 * --hex, the full canonical residue in hex.  res64 is the low 64 bits of the
 * canonical residue in [0, M_p) (M_p itself maps to 0).
 *
 * Build: gcc -O2 -o gmp_chain gmp_chain.c -l:libgmp.so.10
 * Usage: gmp_chain <p> <prp|ll|prp3> <iters> <every|list> [--hex]
 *        list = comma separated iteration numbers, every = a single number N
 *        meaning every N iterations (and the last one).
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef struct { int alloc; int size; uint64_t* d; } mpz_struct;
typedef mpz_struct mpz_t[1];
void __gmpz_init(mpz_struct*);
void __gmpz_clear(mpz_struct*);
void __gmpz_set_ui(mpz_struct*, unsigned long);
void __gmpz_mul(mpz_struct*, const mpz_struct*, const mpz_struct*);
void __gmpz_mul_ui(mpz_struct*, const mpz_struct*, unsigned long);
void __gmpz_add(mpz_struct*, const mpz_struct*, const mpz_struct*);
void __gmpz_sub(mpz_struct*, const mpz_struct*, const mpz_struct*);
void __gmpz_sub_ui(mpz_struct*, const mpz_struct*, unsigned long);
void __gmpz_add_ui(mpz_struct*, const mpz_struct*, unsigned long);
void __gmpz_setbit(mpz_struct*, unsigned long);
int __gmpz_cmp(const mpz_struct*, const mpz_struct*);
int __gmpz_cmp_ui(const mpz_struct*, unsigned long);
void __gmpz_tdiv_q_2exp(mpz_struct*, const mpz_struct*, unsigned long);
void __gmpz_tdiv_r_2exp(mpz_struct*, const mpz_struct*, unsigned long);
unsigned long __gmpz_get_ui(const mpz_struct*);
char* __gmpz_get_str(char*, int, const mpz_struct*);

static mpz_t M, hi, lo;

/* x <- x mod M_p for 0 <= x < 2^(2p+2), using 2^p == 1 (mod M_p). */
static void mod_mersenne(mpz_struct* x, unsigned long p) {
    for (int r = 0; r < 2; ++r) {
        __gmpz_tdiv_q_2exp(hi, x, p);
        __gmpz_tdiv_r_2exp(lo, x, p);
        __gmpz_add(x, hi, lo);
    }
    while (__gmpz_cmp(x, M) >= 0) __gmpz_sub(x, x, M);
}

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s <p> <prp|ll|prp3> <iters> <every|list> [--hex]\n", argv[0]);
        return 1;
    }
    unsigned long p = strtoul(argv[1], NULL, 10);
    const char* mode = argv[2];
    unsigned long iters = strtoul(argv[3], NULL, 10);
    int hex = (argc > 5 && strcmp(argv[5], "--hex") == 0);
    int is_ll = strcmp(mode, "ll") == 0, is_prp3 = strcmp(mode, "prp3") == 0;
    unsigned long every = 0;
    unsigned long list[4096]; int nlist = 0;
    if (strchr(argv[4], ',')) {
        char* s = strdup(argv[4]);
        for (char* t = strtok(s, ","); t && nlist < 4096; t = strtok(NULL, ",")) list[nlist++] = strtoul(t, NULL, 10);
    } else {
        every = strtoul(argv[4], NULL, 10);
    }
    __gmpz_init(M); __gmpz_init(hi); __gmpz_init(lo);
    __gmpz_set_ui(M, 0); __gmpz_setbit(M, p); __gmpz_sub_ui(M, M, 1);
    mpz_t x; __gmpz_init(x);
    __gmpz_set_ui(x, is_ll ? 4 : 3);
    for (unsigned long k = 1; k <= iters; ++k) {
        __gmpz_mul(x, x, x);
        if (is_prp3) __gmpz_mul_ui(x, x, 3);
        mod_mersenne(x, p);
        if (is_ll) {
            if (__gmpz_cmp_ui(x, 2) < 0) __gmpz_add(x, x, M);
            __gmpz_sub_ui(x, x, 2);
        }
        int emit = 0;
        if (every) emit = (k % every == 0) || k == iters;
        else for (int i = 0; i < nlist; ++i) if (list[i] == k) emit = 1;
        if (emit) {
            if (__gmpz_cmp(x, M) == 0) __gmpz_set_ui(x, 0);
            printf("iter %lu res64 %016lx", k, __gmpz_get_ui(x));
            if (hex) {
                char* s = __gmpz_get_str(NULL, 16, x);
                printf(" hex %s", s);
                free(s);
            }
            printf("\n");
            fflush(stdout);
        }
    }
    return 0;
}
