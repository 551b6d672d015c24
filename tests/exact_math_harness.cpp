// Host build of the step kernel's exact-arithmetic helpers (poe2d_math.cuh),
// loaded by tests/test_exact_math.py: each entry point applies one helper to
// n operand tuples.  Compiled with -ffp-contract=off like the device code's
// -fmad=false, so every operation rounds as written.
#include "poe2d_math.cuh"

extern "C" {

void d4_many(const float *a, const float *b, const float *c, const float *d, long n, float h, float *exact,
             float *fast)
{
    const poe::Div24 q = poe::make_div24(h);
    for (long i = 0; i < n; ++i) {
        exact[i] = poe::d4_exact(a[i], b[i], c[i], d[i], q);
        fast[i] = poe::d4_fast(a[i], b[i], c[i], d[i], q);
    }
}

void div_by_many(const float *a, const float *b, long n, float *out)
{
    for (long i = 0; i < n; ++i) out[i] = poe::div_by(a[i], b[i], 1.0f / b[i]);
}

void div24_info(float h, float *D, float *Dl, int *few_bits)
{
    const poe::Div24 q = poe::make_div24(h);
    *D = q.D;
    *Dl = q.Dl;
    *few_bits = q.few_bits;
}

void sxz_many(const float *s, const float *c33, const float *S, long n, float dt, float *out)
{
    for (long i = 0; i < n; ++i) out[i] = poe::sxz_exact(s[i], c33[i], S[i], dt);
}

void sxx_szz_many(const float *l, const float *m, const float *g1, const float *g2, const float *al, const float *p,
                  long n, float *sxx, float *szz)
{
    for (long i = 0; i < n; ++i) poe::sxx_szz_exact(l[i], m[i], g1[i], g2[i], al[i], p[i], sxx[i], szz[i]);
}
}
