// The layer-parallel form of the full-matrix (implicit-scheme 9) column
// solve, for batches with too few columns to fill the GPU.  Included by
// sg_stage.cu after sg_vic.cuh, inside its anonymous namespace.
//
// Reference: the block-Thomas sweep ForwardSweep
// (src/implicit/forward_sweep_impl.h:30-131), the scaled partial-pivot LU
// ludcmp / lubksb (src/math/ludcmp.h:30-95, src/math/lubksb.h:24-71), the
// back substitution and the Woodbury step of the two corrected-PE wall rows
// (src/implicit/vic_kernels.h:100-160).  The system, its right-hand sides
// (du / dt_corr and the two Woodbury unit vectors) and the Woodbury step are
// the serial solve's (vic_solve_kernel); the order of elimination is not.
//
// Why.  The serial sweep is a chain of n dependent 5x5 block steps per
// column.  On GB300 an FP64 warp instruction issues once per 64 cycles per
// SM sub-partition, whether it carries one lane or 32, so a batch of 512
// columns (Straka 512x128) keeps 128 of the 608 sub-partitions busy and the
// solve's time is one column's chain.  This form cuts each column into four
// chunks separated by three single separator layers and gives each chunk to
// one 8-lane group of the column's warp:
//
//   1. each group sweeps its chunk top-down (block Thomas) with the left
//      separator's coupling -B_s as five more right-hand sides:
//        x_i = y_i - C'_i x_{i+1} + V'_i x_L          (x_L the left separator)
//   2. and runs back up the chunk to express every layer in the separators:
//        x_i = Y_i + E_i x_R + F_i x_L
//        Y_i = y_i - C'_i Y_{i+1},  E_i = -C'_i E_{i+1},  F_i = V'_i - C'_i F_{i+1}
//      from Y_e = y_e, E_e = -C'_e (0 in the last chunk), F_e = V'_e;
//   3. separator p's own row, with x_{sigma-1} and x_{sigma+1} substituted,
//      is a block-tridiagonal row in the separators:
//        (A - B C'_e + C F_s) x_p + (B V'_e) x_{p-1} + (C E_s) x_{p+1}
//            = r - B y_e - C Y_s
//   4. every group solves that 3-row system (the same instructions, so each
//      holds the separators' solution);
//   5. each layer's solution follows in parallel from (Y_i, E_i, F_i);
//   6. the Woodbury step as in the serial solve.
//
// The critical path is about n/4 layers of block steps instead of n, and
// every product is a fused multiply-add (fma(), whatever the unit's
// contraction flag): about 150 FP64 warp instructions per layer, against
// the serial form's 210 per layer with separate multiplies and adds (its
// bitwise parity with the oracle needs them).  Reciprocals are two
// Newton-Raphson steps from an FP32 seed (psw_rcp), and the pivot search
// compares its scaled magnitudes in FP32.  The result is the serial
// solve's to rounding (within 1e-12 relative), not bit for bit.
//
// Failure.  A column whose any check fails (non-finite input or factor,
// a zero row, a pivot below the reference's tolerance 8 * 5 * eps of its
// row scale, a non-finite solution) is marked in the mask, and the serial
// solve (vic_solve_kernel) then solves it from the untouched blocks and
// decides its failure exactly as the reference does.  The form writes only
// its own region (E, F and the mask) and D, Z0, Z1.
#pragma once

constexpr int kPswChunks = 4;  // chunks per column (8-lane groups)

// the form's region of a block (after sg_set_sweep): per interior cell the
// E block, then the F block (25 doubles each, row-major, cell = column * n +
// layer), then one int per column: 1 if the serial solve must redo it
struct PswScratch {
  double *E, *F;
  int* mask;
};

__device__ __forceinline__ PswScratch psw_scratch(const BlockDev& B,
                                                  size_t cells) {
  PswScratch s;
  s.E = B.psw;
  s.F = B.psw + 25 * cells;
  s.mask = reinterpret_cast<int*>(B.psw + kPswDoublesPerCell * cells);
  return s;
}

__device__ __forceinline__ float psw_rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// 1 / x by Newton-Raphson iteration for the reciprocal,
//   r <- r + r (1 - x r),
// which doubles the correct bits per step, from a seed r0 = the FP32
// reciprocal approximation of x's leading 23 mantissa bits, scaled by x's
// exponent with integer operations (relative error below 2^-21); two steps
// give 1 / x within about an ulp.  Four FP64 fused multiply-adds, against
// about nine FP64-pipe instructions for the IEEE division.  Zero,
// subnormal, infinite, NaN and extreme-exponent x take the division.
__device__ __forceinline__ double psw_rcp(double x) {
  const long long b = __double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex < 2 || ex > 2044) return 1.0 / x;
  const unsigned m = 0x3f800000u | (unsigned)((b >> 29) & 0x7fffffll);
  const unsigned rf = __float_as_uint(psw_rcp_approx(__uint_as_float(m)));
  // rf in (0.5, 1]: its float exponent is 126 or 127
  const long long ef = (long long)(rf >> 23);
  const long long r0 = (b & (long long)0x8000000000000000ull) |
                       ((ef + 1919 - ex) << 52) |
                       ((long long)(rf & 0x7fffffu) << 29);
  double r = __longlong_as_double(r0);
  double e = fma(-x, r, 1.0);
  r = fma(r, e, r);
  e = fma(-x, r, 1.0);
  return fma(r, e, r);
}

// a non-negative double as a float for comparisons only: the exponent
// rebased and clamped to the float range, the mantissa truncated
__device__ __forceinline__ float psw_narrow(double ax) {
  const long long b = __double_as_longlong(ax);
  int e = (int)(b >> 52) - 896;
  const unsigned mant = e <= 0 ? 0u : (unsigned)((b >> 29) & 0x7fffffll);
  e = e < 0 ? 0 : (e > 254 ? 254 : e);
  return __uint_as_float(((unsigned)e << 23) | mant);
}

__device__ __forceinline__ double psw_shfl(double v, int src) {
  return __shfl_sync(0xffffffffu, v, src, kVicLanes);
}

// the scaled partial-pivot LU of one group's 5x5 block: lane q < 5 holds
// column q in x; on return x holds column q of the factors (the unit lower
// part below the diagonal), indx the pivot row of every step (the same on
// all lanes of the group), rdq = 1 / u_qq on lane q (lanes q >= 5: x comes
// back with its rows exchanged, and is not used); good is cleared on
// this lane for a non-finite entry, a zero row, a pivot below the
// tolerance or a non-finite factor
__device__ __forceinline__ void psw_lu(double (&x)[5], int (&indx)[5],
                                       double& rdq, bool& good, int q) {
  const bool colane = q < 5;
  unsigned long long mx[5];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    if (colane) good = good && vfinite(x[r]);
    mx[r] = colane ? vbits(fabs(x[r])) : 0ull;
  }
#pragma unroll
  for (int off = 4; off >= 1; off >>= 1)
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      const unsigned long long o =
          __shfl_xor_sync(0xffffffffu, mx[r], off, kVicLanes);
      mx[r] = o > mx[r] ? o : mx[r];
    }
  // the row scales (FP32, carried through the swaps) and their reciprocals
  float sc[5], vv[5];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    sc[r] = psw_narrow(__longlong_as_double((long long)mx[r]));
    good = good && sc[r] > 0.f;
    vv[r] = psw_rcp_approx(sc[r]);
  }
  rdq = 0.;
#pragma unroll
  for (int J = 0; J < 5; ++J) {
    // the pivot: the last row of the largest vv |a_iJ| (lane J's column)
    float best = -1.f;
    int imax = J;
#pragma unroll
    for (int i2 = J; i2 < 5; ++i2) {
      const float d = vv[i2] * psw_narrow(fabs(x[i2]));
      if (d >= best) {
        best = d;
        imax = i2;
      }
    }
    imax = __shfl_sync(0xffffffffu, imax, J, kVicLanes);
    indx[J] = imax;
#pragma unroll
    for (int i2 = J + 1; i2 < 5; ++i2)
      if (imax == i2) {
        // the block's rows (lanes q < 5; lanes q >= 5 swap too, and their
        // callers keep the unpermuted right-hand side aside)
        const double t = x[J];
        x[J] = x[i2];
        x[i2] = t;
        float f = vv[J];
        vv[J] = vv[i2];
        vv[i2] = f;
        f = sc[J];
        sc[J] = sc[i2];
        sc[i2] = f;
      }
    const double piv = psw_shfl(x[J], J);
    const double dinv = psw_rcp(piv);
    if (q == J) {
      rdq = dinv;
      // the reference's pivot tolerance: |u_JJ| / scale_J <= 8 n eps
      good = good && vfinite(dinv) &&
             !(psw_narrow(fabs(piv)) <= 8.8817842e-15f * sc[J]);
    }
    if (J < 4) {
      double l[5];
#pragma unroll
      for (int i2 = J + 1; i2 < 5; ++i2) {
        l[i2] = psw_shfl(x[i2], J) * dinv;
        if (q == J) x[i2] = l[i2];
      }
      if (colane && q > J) {
#pragma unroll
        for (int i2 = J + 1; i2 < 5; ++i2) x[i2] = fma(-l[i2], x[J], x[i2]);
      }
    }
  }
  if (colane) {
#pragma unroll
    for (int r = 0; r < 5; ++r) good = good && vfinite(x[r]);
  }
}

// lubksb on one right-hand side v with a group's staged factors lu (row
// major) and diagonal reciprocals rd
__device__ __forceinline__ void psw_lubksb(double (&v)[5], const int (&indx)[5],
                                           const double* lu, const double* rd) {
#pragma unroll
  for (int rr = 0; rr < 5; ++rr) {
    const int ip = indx[rr];
#pragma unroll
    for (int k = rr + 1; k < 5; ++k)
      if (ip == k) {
        const double t = v[k];
        v[k] = v[rr];
        v[rr] = t;
      }
  }
#pragma unroll
  for (int rr = 1; rr < 5; ++rr)
#pragma unroll
    for (int jj = 0; jj < rr; ++jj) v[rr] = fma(-lu[rr * 5 + jj], v[jj], v[rr]);
#pragma unroll
  for (int rr = 4; rr >= 0; --rr) {
#pragma unroll
    for (int jj = rr + 1; jj < 5; ++jj) v[rr] = fma(-lu[rr * 5 + jj], v[jj], v[rr]);
    v[rr] = v[rr] * rd[rr];
  }
}

struct PswSmem {
  double lu[kPswChunks][25];          // each group's factors
  double rd[kPswChunks][5];
  double red[kPswChunks - 1][4][25];  // separator rows: A^, B^, C^, r^ (15)
  double cpp[kPswChunks][kPswChunks - 1][25];  // the reduced sweep's C''
  double xs[kPswChunks][kPswChunks - 1][15];   // the separators' solution
};

// t <- t - M v for a 5x5 row-major M (all lanes hold M)
__device__ __forceinline__ void psw_sub_mv(double (&t)[5], const double* M,
                                           const double (&v)[5]) {
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    double a = t[r];
#pragma unroll
    for (int k = 0; k < 5; ++k) a = fma(-M[r * 5 + k], v[k], a);
    t[r] = a;
  }
}

// one warp per column: grid (columns, blocks), 32 threads.
// BLK32 false: the FP64-assembled blocks with the partitioned form on
// (sg_set_sweep), every column; its region holds E, F and the mask.
// BLK32 true: the FP32-assembled blocks' columns that the refined solve
// (or the FP32 solve) left to the FP64 solve (mask 1), from their FP32
// blocks widened; E and F go to the FP64 A and B slots, which such blocks
// leave free by then.  A column it solves gets mask 3 (done), one it
// cannot mask 2 (the serial FP64 solve takes it, without counting it again)
template <bool BLK32>
__global__ void __launch_bounds__(32)
    vic_psolve_kernel(const BlockDev* __restrict__ tab, StageParams p) {
  __shared__ PswSmem sm;
  const BlockDev& Bk = tab[blockIdx.y];
  if (!Bk.implicit || Bk.implicit == 1) return;
  if (BLK32 ? !Bk.implicit_f32 : (Bk.implicit_f32 || !Bk.psw)) return;
  const VicScratch S = vic_scratch(Bk);
  const int n = Bk.nc1 - 2 * Bk.ng;
  const size_t ncol = S.cells / n;
  const size_t col = blockIdx.x;
  if (col >= ncol || n < kPswMinLayers) return;
  const unsigned full = 0xffffffffu;
  PswScratch W;
  int* maskp;
  const float *A32 = nullptr, *B32 = nullptr, *C32 = nullptr;
  if (BLK32) {
    const VicScratch32 F32 = vic_scratch32(Bk, S, n);
    maskp = F32.mask + col;
    if (*maskp != 1) return;  // uniform over the warp
    W.E = S.A;
    W.F = S.B;
    A32 = F32.A + col * n * kBlk32;
    B32 = F32.B + col * n * kBlk32;
    C32 = F32.C + col * n * kBlk32;
    if (threadIdx.x == 0) count_fp64_column(p, blockIdx.y);
  } else {
    W = psw_scratch(Bk, S.cells);
    maskp = W.mask + col;
  }
  const int bst = BLK32 ? kBlk32 : 25;  // the row of a cell's block
  const int lane = threadIdx.x, g = lane / kVicLanes, q = lane % kVicLanes;
  const bool colane = q < 5;
  // chunks: m = n - 3 layers in four chunks of L or L + 1 layers; chunk g
  // starts at s0, separator g (g < 3) is the layer after it
  const int m = n - (kPswChunks - 1);
  const int Lb = m / kPswChunks, Lr = m % kPswChunks;
  const int L = Lb + (g < Lr ? 1 : 0);
  const int Lmax = Lb + (Lr > 0 ? 1 : 0);
  const int s0 = g * (Lb + 1) + (g < Lr ? g : Lr);
  const double dtc = p.w2 * p.dt[blockIdx.y];
  const double rdtc = 1.0 / dtc;
  const double* A = S.A + col * n * 25;
  const double* Bm = S.B + col * n * 25;
  const double* C = S.C + col * n * 25;
  auto blkA = [&](int e) -> double { return BLK32 ? widen_exact(A32[e]) : A[e]; };
  auto blkB = [&](int e) -> double { return BLK32 ? widen_exact(B32[e]) : Bm[e]; };
  auto blkC = [&](int e) -> double { return BLK32 ? widen_exact(C32[e]) : C[e]; };
  const double* du = S.du + col * n;
  double* D = S.D + col * n * 5;
  double* Z0 = S.Z0 + col * n * 5;
  double* Z1 = S.Z1 + col * n * 5;
  double* E = W.E + col * n * 25;
  double* F = W.F + col * n * 25;
  double* vout = q == 5 ? D : (q == 6 ? Z0 : Z1);

  // the input screen: du of every layer finite
  bool fin = true;
  for (int e = lane; e < 5 * n; e += 32)
    fin = fin && vfinite(du[(size_t)(e / n) * S.cells + (e % n)]);
  bool good = __all_sync(full, fin);

  // ---- 1. the chunk's sweep, top-down ----
  double s[5], sv[5];  // this lane's solution columns of the previous layer
#pragma unroll
  for (int r = 0; r < 5; ++r) s[r] = sv[r] = 0.;
  double b[25];   // the layer's b block (loaded a layer ahead)
  double xa[5], xc[5];  // the layer's column q of a and c (a layer ahead)
  {
    const int i = s0;
#pragma unroll
    for (int e = 0; e < 25; ++e) b[e] = blkB(i * bst + e);
    if (colane) {
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        xa[r] = blkA(i * bst + r * 5 + q);
        xc[r] = blkC(i * bst + r * 5 + q);
      }
    }
  }
  int indx[5];
  for (int t = 0; t < Lmax; ++t) {
    const bool act = t < L;
    const int i = s0 + (act ? t : L - 1);
    double x[5], c5[5], v5[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      x[r] = colane ? xa[r] : 0.;
      c5[r] = colane ? xc[r] : 0.;
      v5[r] = 0.;
    }
    if (q == 5) {
#pragma unroll
      for (int r = 0; r < 5; ++r) x[r] = du[(size_t)r * S.cells + i] * rdtc;
    }
    if (q == 6 && i == 0) x[4] = 1.;
    if (q == 7 && i == n - 1) x[4] = 1.;
    if (t == 0) {
      // the left separator's coupling moves to the right-hand side
      if (g > 0 && colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) v5[r] = -blkB(i * bst + r * 5 + q);
      }
    } else {
      psw_sub_mv(x, b, s);
      psw_sub_mv(v5, b, sv);
    }
    // the next layer's blocks
    if (t + 1 < L) {
      const int i1 = i + 1;
#pragma unroll
      for (int e = 0; e < 25; ++e) b[e] = blkB(i1 * bst + e);
      if (colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          xa[r] = blkA(i1 * bst + r * 5 + q);
          xc[r] = blkC(i1 * bst + r * 5 + q);
        }
      }
    }
    double rdq;
    bool gl = true;
    double sol[5], solv[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      sol[r] = colane ? c5[r] : x[r];
      solv[r] = v5[r];
    }
    psw_lu(x, indx, rdq, gl, q);
    if (colane) {
#pragma unroll
      for (int r = 0; r < 5; ++r) sm.lu[g][r * 5 + q] = x[r];
      sm.rd[g][q] = rdq;
    }
    __syncwarp();
    psw_lubksb(sol, indx, sm.lu[g], sm.rd[g]);
    psw_lubksb(solv, indx, sm.lu[g], sm.rd[g]);
#pragma unroll
    for (int r = 0; r < 5; ++r) gl = gl && vfinite(sol[r]) && vfinite(solv[r]);
    if (act) {
      good = good && gl;
      if (colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          E[i * 25 + r * 5 + q] = sol[r];   // C'_i
          F[i * 25 + r * 5 + q] = solv[r];  // V'_i
        }
      } else {
#pragma unroll
        for (int r = 0; r < 5; ++r) vout[i * 5 + r] = sol[r];  // y_i
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        s[r] = sol[r];
        sv[r] = solv[r];
      }
    }
    __syncwarp();
  }
  // the chunk's last layer: C'_e, V'_e (lanes < 5), y_e (lanes >= 5)
  double cpe[5], vpe[5];
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    cpe[r] = s[r];
    vpe[r] = sv[r];
  }

  // ---- 2. back up the chunk: x_i = Y_i + E_i x_R + F_i x_L ----
  const bool last = g == kPswChunks - 1;
  double ec[5], fc[5];  // column q of E and F of the layer below (lanes < 5);
                        // ec holds Y (lanes >= 5)
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    ec[r] = colane ? (last ? 0. : -cpe[r]) : cpe[r];
    fc[r] = colane ? vpe[r] : 0.;
  }
  {
    const int e = s0 + L - 1;
    if (colane) {
#pragma unroll
      for (int r = 0; r < 5; ++r) E[e * 25 + r * 5 + q] = ec[r];
    }
  }
  double cp[25];  // C'_i of the layer (loaded a layer ahead)
  {
    const int i = s0 + (L >= 2 ? L - 2 : 0);
#pragma unroll
    for (int k = 0; k < 25; ++k) cp[k] = E[i * 25 + k];
  }
  __syncwarp();
  for (int t = Lmax - 2; t >= 0; --t) {
    const bool act = t <= L - 2;
    const int i = s0 + (act ? t : 0);
    double f5[5];
#pragma unroll
    for (int r = 0; r < 5; ++r)
      f5[r] = colane ? F[i * 25 + r * 5 + q] : vout[i * 5 + r];
    double ne[5], nf[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      double a = 0., c = f5[r];
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        a = fma(-cp[r * 5 + k], ec[k], a);
        c = fma(-cp[r * 5 + k], colane ? fc[k] : ec[k], c);
      }
      ne[r] = a;
      nf[r] = c;
    }
    // lanes < 5: E_i = -C'_i E_{i+1}, F_i = V'_i - C'_i F_{i+1};
    // lanes >= 5: Y_i = y_i - C'_i Y_{i+1} (in nf)
    __syncwarp();  // every lane has read C'_i before E_i replaces it
    if (t >= 1) {
      const int i1 = s0 + (t - 1 <= L - 2 ? t - 1 : 0);
#pragma unroll
      for (int k = 0; k < 25; ++k) cp[k] = E[i1 * 25 + k];
    }
    if (act) {
      if (colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          E[i * 25 + r * 5 + q] = ne[r];
          F[i * 25 + r * 5 + q] = nf[r];
          ec[r] = ne[r];
          fc[r] = nf[r];
        }
      } else {
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          vout[i * 5 + r] = nf[r];
          ec[r] = nf[r];
        }
      }
    }
    __syncwarp();
  }
  // ec, fc: E_s, F_s of the chunk's first layer (lanes < 5), Y_s (ec,
  // lanes >= 5)

  // ---- 3. the separators' rows (group p: separator p, after its chunk) ----
  double es1[5], fs1[5];  // chunk p + 1's first-layer terms
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    es1[r] = __shfl_down_sync(full, ec[r], kVicLanes);
    fs1[r] = __shfl_down_sync(full, fc[r], kVicLanes);
  }
  if (!last) {
    const int sg = s0 + L;
    double bs[25], cs[25];
#pragma unroll
    for (int k = 0; k < 25; ++k) {
      bs[k] = blkB(sg * bst + k);
      cs[k] = blkC(sg * bst + k);
    }
    if (colane) {
      double ah[5], bh[5], ch[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        double a = blkA(sg * bst + r * 5 + q), bb = 0., c = 0.;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
          a = fma(-bs[r * 5 + k], cpe[k], a);
          a = fma(cs[r * 5 + k], fs1[k], a);
          bb = fma(bs[r * 5 + k], vpe[k], bb);
          c = fma(cs[r * 5 + k], es1[k], c);
        }
        ah[r] = a;
        bh[r] = bb;
        ch[r] = c;
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        sm.red[g][0][r * 5 + q] = ah[r];
        sm.red[g][1][r * 5 + q] = bh[r];
        sm.red[g][2][r * 5 + q] = ch[r];
      }
    } else {
      double rh[5];
#pragma unroll
      for (int r = 0; r < 5; ++r)
        rh[r] = q == 5 ? du[(size_t)r * S.cells + sg] * rdtc : 0.;
      psw_sub_mv(rh, bs, cpe);   // - B y_e
      psw_sub_mv(rh, cs, es1);   // - C Y_s
#pragma unroll
      for (int r = 0; r < 5; ++r) sm.red[g][3][(q - 5) * 5 + r] = rh[r];
    }
  }
  __syncwarp();

  // ---- 4. the separators' system, in every group ----
  double yy[kPswChunks - 1][5];
  {
#pragma unroll
    for (int r = 0; r < 5; ++r) s[r] = 0.;
#pragma unroll
    for (int pp = 0; pp < kPswChunks - 1; ++pp) {
      double x[5], c5[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        x[r] = colane ? sm.red[pp][0][r * 5 + q]
                      : sm.red[pp][3][(q - 5) * 5 + r];
        c5[r] = colane ? sm.red[pp][2][r * 5 + q] : 0.;
      }
      if (pp > 0) psw_sub_mv(x, sm.red[pp][1], s);
      double rdq;
      bool gl = true;
      double sol[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) sol[r] = colane ? c5[r] : x[r];
      psw_lu(x, indx, rdq, gl, q);
      __syncwarp();
      if (colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) sm.lu[g][r * 5 + q] = x[r];
        sm.rd[g][q] = rdq;
      }
      __syncwarp();
      psw_lubksb(sol, indx, sm.lu[g], sm.rd[g]);
#pragma unroll
      for (int r = 0; r < 5; ++r) gl = gl && vfinite(sol[r]);
      good = good && gl;
      if (colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) sm.cpp[g][pp][r * 5 + q] = sol[r];
      }
#pragma unroll
      for (int r = 0; r < 5; ++r) {
        s[r] = sol[r];
        yy[pp][r] = sol[r];
      }
    }
    __syncwarp();
    // back substitution (lanes >= 5: their right-hand side)
    double xn[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) xn[r] = yy[kPswChunks - 2][r];
    if (!colane) {
#pragma unroll
      for (int r = 0; r < 5; ++r)
        sm.xs[g][kPswChunks - 2][(q - 5) * 5 + r] = xn[r];
    }
#pragma unroll
    for (int pp = kPswChunks - 3; pp >= 0; --pp) {
      double xv[5];
#pragma unroll
      for (int r = 0; r < 5; ++r) xv[r] = yy[pp][r];
      psw_sub_mv(xv, sm.cpp[g][pp], xn);
#pragma unroll
      for (int r = 0; r < 5; ++r) xn[r] = xv[r];
      if (!colane) {
#pragma unroll
        for (int r = 0; r < 5; ++r) sm.xs[g][pp][(q - 5) * 5 + r] = xn[r];
      }
    }
  }
  __syncwarp();

  // ---- 5. every layer from the separators ----
  {
    double xr[15], xl[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) {
      xr[k] = last ? 0. : sm.xs[g][last ? 0 : g][k];
      xl[k] = g == 0 ? 0. : sm.xs[g][g > 0 ? g - 1 : 0][k];
    }
    for (int t = q; t < L; t += kVicLanes) {
      const int i = s0 + t;
      double e25[25], f25[25];
#pragma unroll
      for (int k = 0; k < 25; ++k) {
        e25[k] = last ? 0. : E[i * 25 + k];
        f25[k] = g == 0 ? 0. : F[i * 25 + k];
      }
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        double* out = v == 0 ? D : (v == 1 ? Z0 : Z1);
#pragma unroll
        for (int r = 0; r < 5; ++r) {
          double a = out[i * 5 + r];
#pragma unroll
          for (int k = 0; k < 5; ++k) {
            a = fma(e25[r * 5 + k], xr[v * 5 + k], a);
            a = fma(f25[r * 5 + k], xl[v * 5 + k], a);
          }
          out[i * 5 + r] = a;
        }
      }
    }
    // the separator after this chunk
    if (!last && !colane) {
      const int sg = s0 + L;
#pragma unroll
      for (int r = 0; r < 5; ++r)
        vout[sg * 5 + r] = sm.xs[g][last ? 0 : g][(q - 5) * 5 + r];
    }
  }
  __syncwarp();

  // ---- 6. the Woodbury step of the two wall rows, as the serial solve ----
  good = __all_sync(full, good);
  if (good) {
    VicK K0 = vic_krows(Bk, n, 0), K1 = vic_krows(Bk, n, n - 1);
    const double k0 = -K0.t0 / dtc, k1 = -K1.t1 / dtc;
    const int a0 = 2, a1 = n - 3;
    const double m00 = 1. + k0 * Z0[a0 * 5], m01 = k0 * Z1[a0 * 5];
    const double m10 = k1 * Z0[a1 * 5], m11 = 1. + k1 * Z1[a1 * 5];
    const double r0 = k0 * D[a0 * 5], r1 = k1 * D[a1 * 5];
    const double det = m00 * m11 - m01 * m10;
    const double al0 = (m11 * r0 - m01 * r1) / det;
    const double al1 = (m00 * r1 - m10 * r0) / det;
    __syncwarp();
    bool f = true;
    for (int e = lane; e < 5 * n; e += 32) {
      double d = D[e];
      d = fma(-Z0[e], al0, d);
      d = fma(-Z1[e], al1, d);
      D[e] = d;
      f = f && vfinite(d);
    }
    good = __all_sync(full, f);
  }
  if (lane == 0) {
    if (BLK32) {
      *maskp = good ? 3 : 2;
    } else {
      // (a column the reference's serial order would solve the same way:
      // not its FP64 retry, so not in the monitor's count)
      *maskp = good ? 0 : 1;
      if (!good) atomicAdd(&p.fallbacks[blockIdx.y], 1ull);
    }
  }
}
