/*
 * Ticket order of the ordered large-world solve (large_world.cuh): tickets
 * (pass p, row r) for passes 0 .. P-1 over R rows, sorted by the key p S + r
 * with ties by p, S the pass skew.  Host and device.
 */
#pragma once

namespace shapes {

/* Tickets of passes 0 .. P-1 over R rows, ordered by key p S + r (ties by p):
 * the number of tickets with key < K. */
__host__ __device__ __forceinline__ long long lw_keys_before(long long K, int P, int S, int R) {
  long long n = 0;
  for (int p = 0; p < P; ++p) {
    const long long x = K - (long long)p * S;
    n += x <= 0 ? 0 : (x >= R ? R : x);
  }
  return n;
}

/* Ticket t (0 <= t < P R) -> (pass index p, row r) in key order. */
__host__ __device__ __forceinline__ void lw_ticket(long long t, int P, int S, int R, int& p_out, int& r_out) {
  long long lo = 0, hi = (long long)(P - 1) * S + R; /* largest K with keys_before(K) <= t, in [lo, hi) */
  while (hi - lo > 1) {
    const long long mid = (lo + hi) >> 1;
    if (lw_keys_before(mid, P, S, R) <= t) lo = mid;
    else hi = mid;
  }
  long long j = t - lw_keys_before(lo, P, S, R);
  p_out = 0;
  r_out = 0;
  for (int p = 0; p < P; ++p) {
    const long long r = lo - (long long)p * S;
    if (r < 0 || r >= R) continue;
    if (j == 0) {
      p_out = p;
      r_out = (int)r;
      return;
    }
    --j;
  }
}

}  // namespace shapes
