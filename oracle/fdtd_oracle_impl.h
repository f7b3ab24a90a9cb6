/*
 * Body of the CPU oracle, included once per precision by fdtd_oracle.c with
 *   REAL      the field type (float or double)
 *   SUF(x)    the symbol suffix (x##_f32 / x##_f64)
 *   NARROW(v) rounding of a double result back to REAL
 *
 * TEST INFRASTRUCTURE: the oracle checks the CUDA engine; nothing in the product links it.
 *
 * Each sub-step is a plain loop over full volumes in the reference's order
 * (meep_gpu/driver.py FdtdDriver.step :3419-3596), the reference's array-path
 * arithmetic restated operation for operation:
 *   step_B / step_D      meep_gpu/stepping.py:333 / :463, curl association
 *                        ((g1s - g1) + g2) - g2s (_curl_from_operands :2265), ghost
 *                        rules _shift_up :2423 / _shift_down :2485, masks
 *                        _mask_non_owned_cells :2589, PML forms _apply_pml_update
 *                        :2629 and _apply_dsig_only_update :2662 chosen per cell by
 *                        the chunk membership (_apply_curl_regions :2705)
 *   zero_metal_B/D       stepping.py:3120 / :3093
 *   update_H / update_E  stepping.py:1216 / :1243 with _apply_constitutive_pml :2991
 *                        and MEEP's start of H (separate_h_from_b :2789)
 *   source deposit       sources.py _deposit :1357 (double subtract, one rounding);
 *                        magnetic sources into B right after step_B (driver.py:3534)
 *   update_P             dispersion.py PolarizationState.update :689
 *   conductivity         stepping.py _apply_conductive_update :2828 (no PML) and
 *                        _apply_conductive_pml_update :2844 (the four conductive forms
 *                        on the dsig / dsigu memberships of the chunks that keep the
 *                        component's conductivity, the lossless forms elsewhere)
 *   DFT accumulation     dft.py _phase_factors :316, _apply_yee_interpolation :352,
 *                        FluxMonitor.update :3031
 */

typedef struct SUF(oracle_pole) {
  REAL two_minus_od, gamma1, omega0dtsqr, gamma1inv;
  const REAL* sigma[3]; /* full volume or NULL (component not driven) */
  REAL* p[3];
  REAL* pp[3];
} SUF(oracle_pole);

typedef struct SUF(oracle_state) {
  int nx, ny, nz;
  int metallic[3];
  REAL dtdx;
  int pml;
  const REAL* kms[2][3];
  const REAL* sinv[2][3];
  const REAL* kps[2][3];
  const unsigned char* member[2][3]; /* chunk membership lines per (lattice, axis) */
  REAL* E[3];
  REAL* D[3];
  REAL* B[3];
  REAL* H[3];   /* full volumes; with no PML pass B's pointers */
  REAL* fwH[3];
  REAL* fwE[3];
  REAL* fuB[3];
  REAL* fuD[3];
  const REAL* inv_eps[3];
  REAL* scratch; /* one volume, the curl */
  REAL* drive[3]; /* W of each component, formed by update_E for update_P */
  int npoles;
  SUF(oracle_pole) poles[8];
  int nsrc;
  const long long* src_cell;
  const int* src_comp;
  int h_separated;
  /* D and B conductivity, [side: 0 B, 1 D][component]; NULL for a lossless component.
   * keeps: full volume, 1 where the cell's chunk keeps the component's conductivity;
   * fcond: the conductive-stage history (PML runs). */
  const REAL* condfac[2][3];
  const REAL* condinv[2][3];
  const unsigned char* keeps[2][3];
  REAL* fcond[2][3];
  /* mirror planes: fold[a] = +1 / -1 (even / odd) folds axis a, whose unfolded count is
   * full[a]; 0: no plane. metallic[a] is the folded axis's far face: on a periodic one
   * (metallic 0) the last slot of the shift-1 components is the second mirror's ghost. */
  int fold[3];
  int full[3];
  /* Bloch phases (a complex run with k != 0, its two parts stepped together): per axis
   * bmode 0 none, 1 copy, 2 negate, 3 the phase (bre, bim); `part` 0 steps the real
   * parts, 1 the imaginary ones; pE / pH the other part's E and H. */
  int bloch;
  int bmode[3];
  REAL bre[3], bim[3];
  int part;
  REAL* pE[3];
  REAL* pH[3];
  /* bit a: axis a is translationally invariant (a 2-D or 1-D run, one periodic cell):
   * a curl partner differenced along it is absent (reference stepping.py:2189
   * curl_presence), and the one-partner forms are dtdx * (g1s - g1) and
   * (-dtdx) * (g2s - g2). */
  int invariant;
} SUF(oracle_state);

/* A curl operand read across a Bloch-phased face at the same stored index (reference
 * stepping.py:2544 _bloch_ghost_operand): this part's word and the other part's times
 * the axis's phase, conjugated for the word below the window (B's forward curl), each
 * product and sum rounded on its own. */
static inline REAL SUF(bloch_word)(const SUF(oracle_state)* s, int axis, int conj, REAL own, REAL other) {
  const int mode = s->bmode[axis];
  if (mode == 2) return -own;
  if (mode != 3) return own;
  const REAL a = s->bre[axis];
  const REAL b = conj ? -s->bim[axis] : s->bim[axis];
  return s->part ? (a * own) + (b * other) : (a * own) - (b * other);
}

static inline long long SUF(lin)(const SUF(oracle_state)* s, int i, int j, int k) {
  return ((long long)i * s->ny + j) * s->nz + k;
}

/* Neighbour one cell up (forward difference) or down (backward): metallic faces read
 * zero, periodic faces wrap. */
static inline REAL SUF(up)(const SUF(oracle_state)* s, const REAL* f, int axis, int i, int j, int k) {
  int idx[3] = {i, j, k};
  const int n[3] = {s->nx, s->ny, s->nz};
  idx[axis] += 1;
  if (idx[axis] == n[axis]) {
    if (s->metallic[axis] || s->fold[axis]) return (REAL)0;
    idx[axis] = 0;
  }
  return f[SUF(lin)(s, idx[0], idx[1], idx[2])];
}

static inline REAL SUF(down)(const SUF(oracle_state)* s, const REAL* f, int axis, int i, int j, int k) {
  int idx[3] = {i, j, k};
  const int n[3] = {s->nx, s->ny, s->nz};
  idx[axis] -= 1;
  if (idx[axis] < 0) {
    if (s->metallic[axis] || s->fold[axis]) return (REAL)0;
    idx[axis] = n[axis] - 1;
  }
  return f[SUF(lin)(s, idx[0], idx[1], idx[2])];
}

/* The split-field curl sub-step of one family: B (forward, half lattice) or D
 * (backward, integer lattice). Component q: first = (q+2)%3 along axis (q+1)%3,
 * second = (q+1)%3 along axis (q+2)%3; dsig = (q+1)%3, dsigu = (q+2)%3. */
static void SUF(curl_family)(SUF(oracle_state)* s, REAL* const target[3], REAL* const src[3],
                             REAL* const fu[3], int backward, REAL* const partner[3]) {
  const int lattice = backward ? 0 : 1;
  const int side = backward ? 1 : 0; /* conductivity side: D steps backward, B forward */
  const int n[3] = {s->nx, s->ny, s->nz};
  for (int q = 0; q < 3; ++q) {
    const int a1 = (q + 1) % 3, a2 = (q + 2) % 3;
    const REAL* g1 = src[a2]; /* first partner: component a2, differenced along a1 */
    const REAL* g2 = src[a1]; /* second partner: component a1, differenced along a2 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n[0]; ++i)
      for (int j = 0; j < n[1]; ++j)
        for (int k = 0; k < n[2]; ++k) {
          const long long c = SUF(lin)(s, i, j, k);
          const REAL g1s = backward ? SUF(down)(s, g1, a1, i, j, k) : SUF(up)(s, g1, a1, i, j, k);
          const REAL g2s = backward ? SUF(down)(s, g2, a2, i, j, k) : SUF(up)(s, g2, a2, i, j, k);
          REAL g1c = g1[c], g2c = g2[c];
          if (s->bloch) {
            /* the same-index operands at index 0 of a phased axis: conj(eikna) below the
             * window for B, eikna above it for D */
            const int at0[3] = {i, j, k};
            if (at0[a1] == 0 && s->bmode[a1]) g1c = SUF(bloch_word)(s, a1, !backward, g1c, partner[a2][c]);
            if (at0[a2] == 0 && s->bmode[a2]) g2c = SUF(bloch_word)(s, a2, !backward, g2c, partner[a1][c]);
          }
          const int have1 = !((s->invariant >> a1) & 1), have2 = !((s->invariant >> a2) & 1);
          REAL curl;
          if (have1 && have2) {
            REAL bracket = g1s - g1c;
            bracket = bracket + g2c;
            bracket = bracket - g2s;
            curl = s->dtdx * bracket;
          } else if (have1) {
            curl = s->dtdx * (g1s - g1c);
          } else if (have2) {
            curl = (-s->dtdx) * (g2s - g2c);
          } else {
            curl = (REAL)0;
          }
          /* mask: cell 0 of every metallic axis where the target's Yee shift is 0 (the
           * wall, or on a folded axis the plane's ghost: reference stepping.py:2589).
           * B (shift 1 on the two transverse axes) has shift 0 only on its own axis q;
           * D has shift 0 on the two transverse axes. */
          const int at[3] = {i, j, k};
          for (int a = 0; a < 3; ++a) {
            const int shift0 = backward ? (a != q) : (a == q);
            if (shift0 && (s->metallic[a] || s->fold[a]) && at[a] == 0) curl = (REAL)0;
            /* the far ghost slot of a folded periodic axis (reference stepping.py:2618) */
            if (!shift0 && s->fold[a] && !s->metallic[a] && at[a] == n[a] - 1) curl = (REAL)0;
          }
          s->scratch[c] = curl;
        }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n[0]; ++i)
      for (int j = 0; j < n[1]; ++j)
        for (int k = 0; k < n[2]; ++k) {
          const long long c = SUF(lin)(s, i, j, k);
          const int at[3] = {i, j, k};
          const REAL curl = s->scratch[c];
          REAL f = target[q][c];
          const REAL* cf = s->condfac[side][q];
          const int lossy = cf != NULL && (!s->pml || s->keeps[side][q][c]);
          if (lossy && !s->pml) {
            REAL g = cf[c] * f;
            g = g - curl;
            f = g * s->condinv[side][q][c];
          } else if (lossy) {
            const REAL fac = cf[c], inv = s->condinv[side][q][c];
            const int sg = s->member[lattice][a1][at[a1]];
            const int su = s->member[lattice][a2][at[a2]];
            const REAL kms = s->kms[lattice][a1][at[a1]], sinv = s->sinv[lattice][a1][at[a1]];
            const REAL kms_u = s->kms[lattice][a2][at[a2]], sinv_u = s->sinv[lattice][a2][at[a2]];
            if (sg) {
              const REAL prev_g = s->fcond[side][q][c];
              REAL g = fac * prev_g;
              g = g - curl;
              g = g * inv;
              s->fcond[side][q][c] = g;
              const REAL inc = g - prev_g;
              if (su) {
                const REAL prev = fu[q][c];
                REAL next = kms * prev;
                next = next + inc;
                next = next * sinv;
                fu[q][c] = next;
                REAL h = kms_u * f;
                h = h + next;
                h = h - prev;
                f = h * sinv_u;
              } else {
                REAL h = kms * f;
                h = h + inc;
                f = h * sinv;
              }
            } else if (su) {
              const REAL prev = fu[q][c];
              REAL next = fac * prev;
              next = next - curl;
              next = next * inv;
              fu[q][c] = next;
              REAL h = kms_u * f;
              h = h + next;
              h = h - prev;
              f = h * sinv_u;
            } else {
              REAL h = fac * f;
              h = h - curl;
              f = h * inv;
            }
          } else if (!s->pml) {
            f = f - curl;
          } else {
            const REAL kms = s->kms[lattice][a1][at[a1]];
            const REAL sinv = s->sinv[lattice][a1][at[a1]];
            if (s->member[lattice][a2][at[a2]]) {
              const REAL prev = fu[q][c];
              REAL next = kms * prev;
              next = next - curl;
              next = next * sinv;
              fu[q][c] = next;
              REAL g = s->kms[lattice][a2][at[a2]] * f;
              g = g + next;
              g = g - prev;
              f = g * s->sinv[lattice][a2][at[a2]];
            } else {
              REAL g = kms * f;
              g = g - curl;
              f = g * sinv;
            }
          }
          target[q][c] = f;
        }
  }
}

/* Hold every component's wall samples at zero: shift-0 axes that are metallic (a
 * folded axis's cell 0 is the plane's ghost, not a wall). */
static void SUF(zero_metal)(SUF(oracle_state)* s, REAL* const f[3], int electric) {
  const int n[3] = {s->nx, s->ny, s->nz};
  for (int q = 0; q < 3; ++q)
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n[0]; ++i)
      for (int j = 0; j < n[1]; ++j)
        for (int k = 0; k < n[2]; ++k) {
          const int at[3] = {i, j, k};
          for (int a = 0; a < 3; ++a) {
            const int shift0 = electric ? (a != q) : (a == q);
            if (shift0 && s->metallic[a] && !s->fold[a] && at[a] == 0) f[q][SUF(lin)(s, i, j, k)] = (REAL)0;
          }
        }
}

/* The sign of component q of a family about the plane normal to axis a (MEEP's
 * phase_shift, reference fields.py:121): E and D odd about their own axis, H and B
 * about the other two, times the plane's phase. */
static int SUF(parity)(const SUF(oracle_state)* s, int q, int a, int electric) {
  const int own = q == a;
  return (electric ? own : !own) ? -s->fold[a] : s->fold[a];
}

/* fill_folded_far_ghosts (reference stepping.py:2092): on a folded periodic axis the
 * last slot of every shift-1 component = parity * the row it images about the second
 * mirror at doubled full, full - n + 2. */
static void SUF(fill_far)(SUF(oracle_state)* s, REAL* const f[3], int electric) {
  const int n[3] = {s->nx, s->ny, s->nz};
  for (int q = 0; q < 3; ++q)
    for (int a = 0; a < 3; ++a) {
      const int shift1 = electric ? (a == q) : (a != q);
      if (!s->fold[a] || s->metallic[a] || !shift1) continue;
      const REAL sign = (REAL)SUF(parity)(s, q, a, electric);
      const int row = s->full[a] - n[a] + 2;
      for (int i = (a == 0 ? n[0] - 1 : 0); i < n[0]; ++i)
        for (int j = (a == 1 ? n[1] - 1 : 0); j < n[1]; ++j)
          for (int k = (a == 2 ? n[2] - 1 : 0); k < n[2]; ++k) {
            int src[3] = {i, j, k};
            src[a] = row;
            f[q][SUF(lin)(s, i, j, k)] = sign * f[q][SUF(lin)(s, src[0], src[1], src[2])];
          }
    }
}

/* fill_symmetry_bc (reference stepping.py:2038): cell 0 = parity * cell 2 on every
 * folded axis where the component's Yee shift is 0, axes in x, y, z order. */
static void SUF(fill_symmetry)(SUF(oracle_state)* s, REAL* const f[3], int electric) {
  const int n[3] = {s->nx, s->ny, s->nz};
  for (int q = 0; q < 3; ++q)
    for (int a = 0; a < 3; ++a) {
      const int shift0 = electric ? (a != q) : (a == q);
      if (!s->fold[a] || !shift0) continue;
      const REAL sign = (REAL)SUF(parity)(s, q, a, electric);
      for (int i = 0; i < (a == 0 ? 1 : n[0]); ++i)
        for (int j = 0; j < (a == 1 ? 1 : n[1]); ++j)
          for (int k = 0; k < (a == 2 ? 1 : n[2]); ++k) {
            int src[3] = {i, j, k};
            src[a] = 2;
            f[q][SUF(lin)(s, i, j, k)] = sign * f[q][SUF(lin)(s, src[0], src[1], src[2])];
          }
    }
}

/* One half of a step: 0 the H half (step_B, magnetic sources, fills, update_H), 1 the E
 * half (step_D, electric sources, fills, update_E, update_P). A Bloch run steps the H
 * halves of both parts, then the E halves. */
void SUF(oracle_half)(SUF(oracle_state)* s, const double* words, int half) {
  const int n[3] = {s->nx, s->ny, s->nz};
  const long long cells = (long long)n[0] * n[1] * n[2];
  if (half == 1) goto e_half;
  /* 1. step_B, 2. magnetic sources (components 3..5, B = NARROW(double(B) - A)),
   * 2b. zero_metal_B */
  SUF(curl_family)(s, s->B, s->E, s->fuB, 0, s->pE);
  for (int p = 0; p < s->nsrc; ++p) {
    if (s->src_comp[p] < 3) continue;
    REAL* b = s->B[s->src_comp[p] - 3];
    const long long c = s->src_cell[p];
    b[c] = NARROW((double)b[c] - words[p]);
  }
  SUF(fill_symmetry)(s, s->B, 0);
  SUF(zero_metal)(s, s->B, 0);
  SUF(fill_far)(s, s->B, 0);
  /* 3. update_H (stored H only under a PML) */
  if (s->pml) {
    if (!s->h_separated) {
      for (int q = 0; q < 3; ++q)
        for (int i = 0; i < n[0]; ++i)
          for (int j = 0; j < n[1]; ++j)
            for (int k = 0; k < n[2]; ++k) {
              const int at[3] = {i, j, k};
              if (!s->member[0][q][at[q]]) continue;
              const long long c = SUF(lin)(s, i, j, k);
              s->H[q][c] = s->B[q][c];
              s->fwH[q][c] = s->B[q][c];
            }
    }
    for (int q = 0; q < 3; ++q)
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n[0]; ++i)
        for (int j = 0; j < n[1]; ++j)
          for (int k = 0; k < n[2]; ++k) {
            const int at[3] = {i, j, k};
            const long long c = SUF(lin)(s, i, j, k);
            if (s->member[0][q][at[q]]) {
              const REAL prev = s->fwH[q][c];
              s->fwH[q][c] = s->B[q][c];
              REAL product = s->kps[0][q][at[q]] * s->fwH[q][c];
              REAL back = s->kms[0][q][at[q]] * prev;
              product = product - back;
              s->H[q][c] = s->H[q][c] + product;
            } else {
              s->H[q][c] = s->B[q][c];
            }
          }
  }
  s->h_separated = 1;
  return;
e_half:
  /* 4. step_D */
  SUF(curl_family)(s, s->D, s->H, s->fuD, 1, s->pH);
  /* 5. electric sources: D = NARROW(double(D) - A) point by point */
  for (int p = 0; p < s->nsrc; ++p) {
    if (s->src_comp[p] >= 3) continue;
    REAL* d = s->D[s->src_comp[p]];
    const long long c = s->src_cell[p];
    d[c] = NARROW((double)d[c] - words[p]);
  }
  /* 6. fill_symmetry_bc_D, 6b. zero_metal_D */
  SUF(fill_symmetry)(s, s->D, 1);
  SUF(zero_metal)(s, s->D, 1);
  SUF(fill_far)(s, s->D, 1);
  /* 7. update_E: W = chi1inv * (D - sum P); E = W, or the own-axis accumulation. */
  for (int q = 0; q < 3; ++q)
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n[0]; ++i)
      for (int j = 0; j < n[1]; ++j)
        for (int k = 0; k < n[2]; ++k) {
          const int at[3] = {i, j, k};
          const long long c = SUF(lin)(s, i, j, k);
          REAL dmp = s->D[q][c];
          for (int m = 0; m < s->npoles; ++m)
            if (s->poles[m].sigma[q] != NULL) dmp = dmp - s->poles[m].p[q][c];
          const REAL w = s->inv_eps[q][c] * dmp;
          if (s->pml && s->member[1][q][at[q]]) {
            const REAL prev = s->fwE[q][c];
            s->fwE[q][c] = w;
            REAL product = s->kps[1][q][at[q]] * w;
            REAL back = s->kms[1][q][at[q]] * prev;
            product = product - back;
            s->E[q][c] = s->E[q][c] + product;
          } else {
            s->E[q][c] = w;
          }
          s->drive[q][c] = w;
        }
  /* 7b. update_P from the W of the step just closed; P_prev <- P, P <- P'. */
  for (int m = 0; m < s->npoles; ++m) {
    SUF(oracle_pole)* pole = &s->poles[m];
    for (int q = 0; q < 3; ++q) {
      if (pole->sigma[q] == NULL) continue;
#pragma omp parallel for schedule(static)
      for (long long c = 0; c < cells; ++c) {
        const REAL pcur = pole->p[q][c];
        REAL acc = pcur * pole->two_minus_od;
        acc = acc - pole->gamma1 * pole->pp[q][c];
        REAL drive = pole->sigma[q][c] * s->drive[q][c];
        drive = pole->omega0dtsqr * drive;
        acc = acc + drive;
        pole->pp[q][c] = pcur;
        pole->p[q][c] = pole->gamma1inv * acc;
      }
    }
  }
}

void SUF(oracle_step)(SUF(oracle_state)* s, const double* words) {
  SUF(oracle_half)(s, words, 0);
  SUF(oracle_half)(s, words, 1);
}

/* Monitor accumulation on a post-increment step: cell-centred samples (x, then y, then
 * z averages on shift-0 axes) times exp(i w t) * scale, E at t = step*dt, H at t - dt/2.
 * comp: 0..2 E, 3..5 H. acc: [ncomp][nfreq][2][cells]. In the float32 oracle the
 * phase is rounded to float32 and the products and sums are float32, as complex64. */
static REAL SUF(sample_at)(const SUF(oracle_state)* s, const REAL* f, const REAL* other, int cp, int i, int j,
                           int k) {
  const int n[3] = {s->nx, s->ny, s->nz};
  int at[3] = {i, j, k};
  REAL sign = (REAL)1;
  for (int a = 0; a < 3; ++a) {
    if (s->fold[a]) {
      /* a folded axis (reference dft.py:1004 folded_axis_sites): site r of a component
       * with Yee shift p sits at doubled -2 + 2r + p; outside the unfolded cell's owned
       * window it is zero, below the plane the image at -d with the component's parity,
       * and at the far wall zero */
      const int q = cp % 3, electric = cp < 3;
      const int p = electric ? (a == q) : (a != q);
      const int periodic = !s->metallic[a];
      const int low = -(s->full[a] - s->full[a] % 2), lattice = 2 * s->full[a];
      int d = -2 + 2 * at[a] + p;
      if (d < low + 2 - p || d > low + lattice - p) {
        if (!periodic) return (REAL)0;
        d += d < low + 2 - p ? lattice : -lattice;
        if (d < low + 2 - p || d > low + lattice - p) return (REAL)0;
      }
      if (d < -p) {
        d = -d;
        sign = sign * (REAL)SUF(parity)(s, q, a, electric);
      }
      at[a] = (d + 2 - p) / 2;
      if (at[a] >= n[a]) {
        if (!periodic) return (REAL)0;
        d = lattice - d; /* the second mirror at doubled full */
        sign = sign * (REAL)SUF(parity)(s, q, a, electric);
        if (d + 2 - p < 0 || (d + 2 - p) / 2 >= n[a]) return (REAL)0;
        at[a] = (d + 2 - p) / 2;
      }
      continue;
    }
    if (at[a] >= n[a] || at[a] < 0) {
      if (s->metallic[a]) return (REAL)0;
      at[a] %= n[a];
      if (at[a] < 0) at[a] += n[a];
    }
  }
  const REAL own = sign * f[SUF(lin)(s, at[0], at[1], at[2])];
  if (!s->bloch) return own;
  /* On a Bloch-phased axis the ladder point r is eikna^count times the stored word, count
   * = floor((r - low) / n), low 1 for a component with Yee shift 0 there (its cell 0
   * stores the owned top point), the powers by repeated products (reference dft.py:927) */
  const int raw[3] = {i, j, k};
  const int q = cp % 3, electric = cp < 3;
  REAL fr = (REAL)1, fi = (REAL)0;
  int any = 0;
  for (int a = 0; a < 3; ++a) {
    if (!s->bmode[a]) continue;
    const int low = (electric ? (a != q) : (a == q)) ? 1 : 0;
    const int shifted = raw[a] - low;
    int count = shifted >= 0 ? shifted / n[a] : -((-shifted + n[a] - 1) / n[a]);
    const REAL br = s->bmode[a] == 2 ? (REAL)-1 : s->bmode[a] == 1 ? (REAL)1 : s->bre[a];
    const REAL bi0 = s->bmode[a] == 3 ? s->bim[a] : (REAL)0;
    const REAL bi = count < 0 ? -bi0 : bi0;
    for (count = count < 0 ? -count : count; count > 0; --count) {
      const REAL nr = fr * br - fi * bi, ni = fr * bi + fi * br;
      fr = nr;
      fi = ni;
      any = 1;
    }
  }
  if (!any) return own;
  const REAL o = other[SUF(lin)(s, at[0], at[1], at[2])];
  return s->part ? (fr * own) + (fi * o) : (fr * own) - (fi * o);
}

void SUF(oracle_dft)(const SUF(oracle_state)* s, const int region[6], int ncomp, const int* comp,
                     int nfreq, const double* omega, double scale, double dt, long long step,
                     REAL* acc) {
  const int rx = region[1] - region[0], ry = region[3] - region[2], rz = region[5] - region[4];
  const long long cells = (long long)rx * ry * rz;
  const double t_e = (double)step * dt;
  const double t_h = t_e - 0.5 * dt;
  for (int q = 0; q < ncomp; ++q) {
    const int cp = comp[q];
    const int axis = cp % 3;
    const int electric = cp < 3;
    const REAL* f = electric ? s->E[axis] : s->H[axis];
    const REAL* other = electric ? s->pE[axis] : s->pH[axis];
    int avg[3];
    for (int a = 0; a < 3; ++a) avg[a] = electric ? (a != axis) : (a == axis);
#pragma omp parallel for schedule(static)
    for (long long cell = 0; cell < cells; ++cell) {
      const int rk = (int)(cell % rz), rj = (int)((cell / rz) % ry), ri = (int)(cell / ((long long)ry * rz));
      const int i = region[0] + ri, j = region[2] + rj, k = region[4] + rk;
      REAL v[2][2];
      for (int b = 0; b < 2; ++b)
        for (int a = 0; a < 2; ++a) {
          if ((a && !avg[1]) || (b && !avg[2])) { v[b][a] = 0; continue; }
          const REAL f0 = SUF(sample_at)(s, f, other, cp, i, j + a, k + b);
          if (avg[0]) {
            const REAL f1 = SUF(sample_at)(s, f, other, cp, i + 1, j + a, k + b);
            v[b][a] = (REAL)0.5 * (f0 + f1);
          } else {
            v[b][a] = f0;
          }
        }
      REAL r0 = avg[1] ? (REAL)0.5 * (v[0][0] + v[0][1]) : v[0][0];
      REAL value = r0;
      if (avg[2]) {
        const REAL r1 = avg[1] ? (REAL)0.5 * (v[1][0] + v[1][1]) : v[1][0];
        value = (REAL)0.5 * (r0 + r1);
      }
      const double t = electric ? t_e : t_h;
      for (int fr = 0; fr < nfreq; ++fr) {
        const double x = t * omega[fr];
        const REAL pr = NARROW(cos(x) * scale);
        const REAL pi = NARROW(sin(x) * scale);
        REAL* re = acc + (((long long)q * nfreq + fr) * 2) * cells + cell;
        REAL* im = re + cells;
        *re = *re + pr * value;
        *im = *im + pi * value;
      }
    }
  }
}
