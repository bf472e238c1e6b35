// ResolveContacts (contact.go:204-445) for worlds whose bodies do not fit the
// shared-memory slot of k_resolve (hundreds to thousands of bodies).
//
// One warp per world, or one per two worlds (16 lanes each).  Body and
// contact working rows live in global memory (L2-resident at these sizes).
// The argmax over a world's contacts is a lane-strided scan (four interleaved
// chains per lane) and the first-maximum butterfly of k_resolve.  After
// prepareContacts every body gets the list of its contacts (counting sort by
// body, in global memory), so the update after each resolved contact visits
// only the contacts of the two resolved bodies instead of all C: the
// reference's loop over every contact skips the others, so the visited set
// and each contact's arithmetic are the same (penetration_update /
// velocity_update), and the float64 form stays bit-identical.  The order of
// the visits does not matter: each contact's update reads only its own rows
// and the resolved contact's broadcast changes.
#pragma once
#include "cz_resolve.cuh"

namespace cz {

// Visit every contact of bodies d0 and d1 once (lists adj[off[b] .. end[b]))
// with the G lanes of a group.
template <int G, class R, class W, class F>
__device__ __forceinline__ void for_pair_contacts(const RCtx<R, W>& x, const int* __restrict__ adj, const int* off,
                                                  const int* end, int d0, int d1, int gl, F f) {
  const int o0 = off[d0], l0 = end[d0] - o0;
  const int o1 = d1 >= 0 ? off[d1] : 0, l1 = d1 >= 0 ? end[d1] - o1 : 0;
  for (int e = gl; e < l0 + l1; e += G) {
    int k;
    if (e < l0) {
      k = adj[o0 + e];
    } else {
      k = adj[o1 + e - l0];
      const int bb = x.cb[k];
      if (body0_of(bb) == d0 || body1_of(bb) == d0) continue;  // visited in d0's list
    }
    f(k);
  }
}

// The lane's first maximum of key_of(row[k], 0.01) over its contacts k = gl,
// gl + G, ...: four interleaved running maxima (four independent compare
// chains instead of one), each keeping its first maximum, merged by key and
// then the smaller index.  The result is what one in-order scan of the
// lane's contacts finds.
template <int G, class R, class W>
__device__ __forceinline__ void lane_first_max(const RCtx<R, W>& x, int row, int C, int gl,
                                               decltype(key_of((R)0, (R)0))& best, int& bidx) {
  using K = decltype(key_of((R)0, (R)0));
  K b[4];
  int ix[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    b[q] = 0;
    ix[q] = 0x7fffffff;
  }
  int k = gl;
  for (; k + 3 * G < C; k += 4 * G) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const K key = key_of(x.Cf(row, k + G * q), (R)0.01);
      if (key > b[q]) {
        b[q] = key;
        ix[q] = k + G * q;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) {  // at most three contacts left
    const int kq = k + G * q;
    if (kq < C) {
      const K key = key_of(x.Cf(row, kq), (R)0.01);
      if (key > b[q]) {
        b[q] = key;
        ix[q] = kq;
      }
    }
  }
#pragma unroll
  for (int q = 1; q < 4; ++q) {
    if (b[q] > b[0] || (b[q] == b[0] && ix[q] < ix[0])) {
      b[0] = b[q];
      ix[0] = ix[q];
    }
  }
  best = b[0];
  bidx = ix[0];
}

// One warp, 32 / G worlds of the large-world list (world blockIdx.x * 32 / G
// + group), G lanes each.  With G = 16 the two worlds of a warp run their
// iterations in lockstep, so the sequential part of each iteration (the
// leader's float64 island arithmetic) is issued once for both.  Control flow
// is uniform across the warp: a group whose world is missing or finished
// keeps taking part in the warp-wide shuffles and barriers with its `run`
// flag cleared.
template <class R, class W, int G>
__global__ void __launch_bounds__(32) k_resolve_big(BatchView<R> v, R dt) {
  constexpr int NG = 32 / G;
  __shared__ R bcs[NG][16];
  const int lane = threadIdx.x;
  const int grp = lane / G, gl = lane % G;
  const int wi = blockIdx.x * NG + grp;
  const bool has = wi < v.big_count;
  const int w = has ? v.big_list[wi] : 0;
  const int n = has ? v.body_count[w] : 0;
  const int bstart = has ? v.body_start[w] : 0;
  const long long cst = has ? v.contact_start[w] : 0;
  const long long S = v.nb_pad;
  int C = has ? v.contact_count[w] : 0;
  const int cap = has ? v.contact_cap[w] : 0;
  if (C > cap) C = cap;  // the world is already flagged ST_CAPACITY
  RCtx<R, W> x;
  x.nbs = (int)S;  // row stride of the global body rows
  x.dt = dt;
  x.bw = reinterpret_cast<W*>(v.big_bw) + bstart;
  x.br = v.big_br + bstart;
  x.aw = v.big_aw + bstart;
  x.bc = bcs[grp];
  x.cw = v.work + cst;
  x.cb = v.work_bodies + cst;
  x.cst = v.nc_total;
  x.gmat = v.uniform_material ? nullptr : v.contact + (long long)C_FRIC * v.nc_total + cst;
  x.gst = (long long)(C_REST - C_FRIC) * v.nc_total;
  x.save = x.delta = x.jw = nullptr;
  x.wi = nullptr;
  x.wst = x.jst = 0;
  x.kw = v.kmat + cst * K_ROW;
  const bool active = has && C > 0 && dt > (R)0;  // ResolveContacts guards, contact.go:210-212
  if (has && !active && gl == 0) {
    v.pos_iters[w] = 0;
    v.vel_iters[w] = 0;
    atomicAdd(&v.counters[3], (unsigned long long)C);
  }
  const int na = active ? n : 0;
  const int Ca = active ? C : 0;
  for (int i = gl; i < na; i += G) {
    const long long g = bstart + i;
    x.P(0, i) = (W)v.body[B_PX * S + g];
    x.P(1, i) = (W)v.body[B_PY * S + g];
    x.P(2, i) = (W)v.body[B_PZ * S + g];
    x.P(3, i) = (W)v.body[B_QW * S + g];
    x.P(4, i) = (W)v.body[B_QX * S + g];
    x.P(5, i) = (W)v.body[B_QY * S + g];
    x.P(6, i) = (W)v.body[B_QZ * S + g];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      x.Bf(r, i) = v.body[(B_VX + r) * S + g];
      x.Bf(3 + r, i) = v.body[(B_RX + r) * S + g];
      x.Bf(6 + r, i) = v.body[(B_LX + r) * S + g] * x.dt;  // LastFrameAcceleration * duration
    }
#pragma unroll
    for (int r = 0; r < 9; ++r) x.Bf(9 + r, i) = v.body[(B_IW0 + r) * S + g];
    x.Bf(18, i) = v.body[B_INVM * S + g];
    x.Bf(19, i) = v.body[B_MOTION * S + g];
    x.aw[i] = v.awake[g];
  }
  __syncwarp();
  for (int k = gl; k < Ca; k += G) prepare_contact(x, v, cst + k, k);
  __syncwarp();
  // contact lists per body: count, exclusive scan, fill
  int* off = v.big_off + bstart;
  int* end = v.big_cnt + bstart;  // counts, then the fill cursor, then the list ends
  int* adj = v.big_adj + 2 * cst;
  for (int i = gl; i < na; i += G) end[i] = 0;
  __syncwarp();
  for (int k = gl; k < Ca; k += G) {
    const int bb = x.cb[k];
    atomicAdd(&end[body0_of(bb)], 1);
    if (body1_of(bb) >= 0) atomicAdd(&end[body1_of(bb)], 1);
  }
  __syncwarp();
  const int nmax = __reduce_max_sync(FULL, (unsigned)na);  // the scan's shuffles need every lane
  int carry = 0;
  for (int base = 0; base < nmax; base += G) {
    const int i = base + gl;
    const int c = i < na ? end[i] : 0;
    int s = c;
#pragma unroll
    for (int d = 1; d < G; d <<= 1) {
      const int y = __shfl_up_sync(FULL, s, d, G);
      if (gl >= d) s += y;
    }
    if (i < na) {
      off[i] = carry + s - c;
      end[i] = carry + s - c;
    }
    carry += __shfl_sync(FULL, s, G - 1, G);
  }
  __syncwarp();
  for (int k = gl; k < Ca; k += G) {
    const int bb = x.cb[k];
    adj[atomicAdd(&end[body0_of(bb)], 1)] = k;
    if (body1_of(bb) >= 0) adj[atomicAdd(&end[body1_of(bb)], 1)] = k;
  }
  __syncwarp();
  const int max_it = active ? (v.max_iterations >= 0 ? v.max_iterations : C * v.iter_mult) : 0;
  // ---------------- adjustPositions, contact.go:231-283
  int pos_used = 0;
  bool run = active && max_it > 0;
  while (__any_sync(FULL, run)) {
    auto best = key_of((R)0, (R)0);
    int bidx = 0x7fffffff;
    if (run) lane_first_max<G>(x, W_PEN, C, gl, best, bidx);
    group_first_max<G>(best, bidx);
    if (best == 0) run = false;
    if (run && gl == 0) match_awake(x, x.cb[bidx]);
    __syncwarp();
    apply_position_change<R, W, G>(x, v, bstart, bidx, run, gl);
    __syncwarp();
    if (run) {
      const int rb = x.cb[bidx];
      const int d0 = body0_of(rb), d1 = body1_of(rb);
      for_pair_contacts<G>(x, adj, off, end, d0, d1, gl, [&](int k) { penetration_update(x, k, d0, d1); });
    }
    __syncwarp();
    if (run && ++pos_used >= max_it) run = false;
  }
  for (int k = gl; k < Ca; k += G) friction_prepare(x, k);
  __syncwarp();
  // ---------------- adjustVelocities, contact.go:388-445
  int vel_used = 0;
  run = active && max_it > 0;
  while (__any_sync(FULL, run)) {
    auto best = key_of((R)0, (R)0);
    int bidx = 0x7fffffff;
    if (run) lane_first_max<G>(x, W_DDV, C, gl, best, bidx);
    group_first_max<G>(best, bidx);
    if (best == 0) run = false;
    if (run && gl == 0) {
      match_awake(x, x.cb[bidx]);
      apply_velocity_change<R, W, false>(x, v, w, bidx);
    }
    __syncwarp();
    if (run) {
      const int rb = x.cb[bidx];
      const int d0 = body0_of(rb), d1 = body1_of(rb);
      for_pair_contacts<G>(x, adj, off, end, d0, d1, gl, [&](int k) { velocity_update(x, k, d0, d1); });
    }
    __syncwarp();
    if (run && ++vel_used >= max_it) run = false;
  }
  if (active && gl == 0) {
    v.pos_iters[w] = pos_used;
    v.vel_iters[w] = vel_used;
    atomicAdd(&v.counters[1], (unsigned long long)pos_used);
    atomicAdd(&v.counters[2], (unsigned long long)vel_used);
    atomicAdd(&v.counters[3], (unsigned long long)C);
  }
  if (v.contact_writeback) {
    const long long CS = v.nc_total;
    for (int k = gl; k < Ca; k += G) {
      R* o = v.contact + cst + k;
      o[C_NX * CS] = x.Cf(W_NX, k);
      o[C_NY * CS] = x.Cf(W_NY, k);
      o[C_NZ * CS] = x.Cf(W_NZ, k);
      o[C_PEN * CS] = x.Cf(W_PEN, k);
      v.contact_bodies[cst + k] = x.cb[k];
    }
  }
  for (int i = gl; i < na; i += G) {
    const long long g = bstart + i;
    v.body[B_PX * S + g] = (R)x.P(0, i);
    v.body[B_PY * S + g] = (R)x.P(1, i);
    v.body[B_PZ * S + g] = (R)x.P(2, i);
    v.body[B_QW * S + g] = (R)x.P(3, i);
    v.body[B_QX * S + g] = (R)x.P(4, i);
    v.body[B_QY * S + g] = (R)x.P(5, i);
    v.body[B_QZ * S + g] = (R)x.P(6, i);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      v.body[(B_VX + r) * S + g] = x.Bf(r, i);
      v.body[(B_RX + r) * S + g] = x.Bf(3 + r, i);
    }
#pragma unroll
    for (int r = 0; r < 9; ++r) v.body[(B_IW0 + r) * S + g] = x.Bf(9 + r, i);
    v.body[B_MOTION * S + g] = x.Bf(19, i);
    v.awake[g] = x.aw[i];
  }
}

}  // namespace cz
