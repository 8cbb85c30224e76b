// Host build of the MatrixMarket token parsers of brm_numparse.h (the same
// code the device reader runs), exported so that tests can check the
// conversion against an exact one on many tokens without a GPU.
#include "brm_gen.h"
#include "brm_numparse.h"

namespace {
const uint64_t kPow5Host[brm::kPow5Rows][2] = {BRM_POW5_ROWS};
}

extern "C" {

int brm_parse_int_token(const char *s, int len, long long *out)
{
    return brm::parse_int_tok((const unsigned char *)s, len, out);
}

int brm_parse_real_token(const char *s, int len, double *out)
{
    return brm::parse_real_tok((const unsigned char *)s, len, kPow5Host, out);
}

void brm_parse_real_tokens(const char *buf, const long long *off, const int *len, long long n,
                           double *out, int *status)
{
    for (long long i = 0; i < n; i++)
        status[i] = brm::parse_real_tok((const unsigned char *)buf + off[i], len[i], kPow5Host,
                                        &out[i]);
}
}
