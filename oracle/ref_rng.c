/*
 * ref_rng.c — stand-ins for libc srand()/rand() linked into the reference
 * harness (oracle/_ref) with -Wl,-Bsymbolic, so the reference's
 * calculateForce_AP (UL:1481 srand(time(NULL)), UL:1546 rand()) draws from the
 * same counter-based stream as the GPU path and the C restatement.
 * TEST INFRASTRUCTURE ONLY.
 *
 * Each srand() call starts AP call number `call` (then call += 1); the k-th
 * rand() after it returns philox4x32_10({seed, stream}, {k, call}).x >> 1.
 */
#include <stdint.h>
#include <stdlib.h>

static uint32_t g_seed = 1, g_stream = 0, g_k = 0;
static uint64_t g_next = 0, g_cur = 0;

static void philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3], k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1, n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void ref_rng_set(uint32_t seed, uint32_t stream, uint64_t next_call) {
    g_seed = seed; g_stream = stream; g_next = next_call; g_k = 0;
}
uint64_t ref_rng_calls(void) { return g_next; }

void srand(unsigned int ignored) {
    (void)ignored;
    g_cur = g_next++;
    g_k = 0;
}
int rand(void) {
    uint32_t ctr[4] = {g_k++, (uint32_t)g_cur, (uint32_t)(g_cur >> 32), 0u};
    uint32_t key[2] = {g_seed, g_stream};
    uint32_t out[4];
    philox(ctr, key, out);
    return (int)(out[0] >> 1);
}
