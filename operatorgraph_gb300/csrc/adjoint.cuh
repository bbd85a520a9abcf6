// Adjoint of the derivation (no reference counterpart).
//
// With the discrete derivation frozen -- every IfSizeLess branch, Repeat count,
// discard and the rule of every shape as recorded by the forward pass -- a
// terminal's transform is a smooth function of the continuous inputs: the
// per-axiom parameter blocks (PGA_PT_BLOCK parameters) and the axiom sizes.
// Rotations -- signed permutations, or in the general-frame build the products
// of Rotate's scalar angles -- are changed by no continuous input, so the
// state that carries gradient is a shape's translation t and size s.
//
// Tape: every queued work item stores (parent item or kAxiomLink | axiom,
// child ordinal) in its ext field, every terminal the same pair in termLinks.
// The reverse sweep first visits every terminal, then the levels from the
// deepest up: a record recomputes its creating child from the parent item (or
// the axiom), replays the 1 -> 1 chain to itself, and pushes its gradient
// through the chain and the operator that created it into the parent item's
// accumulator (atomicAdd) and the parameter / axiom-size gradients.
//
// Operator VJPs (o = offset along the split axis a, S = size[a]):
//  Subdivide  size_c = N_c, o_c = -S/2 + sum_{i<c} N_i + N_c/2, N_i = f_i (f > 0)
//             or scale * -f_i (f < 0), scale = (S - sum_abs) / sum_rel.
//  Repeat     size / offset linear in (S, startExt, e2, endExt); extent
//             E = e or S * |e|, the remainder fmod(S, E) = S - k E with k frozen.
//  ComponentSplit  t_f = t + R[:,k] * (+-s_k / 2), face size picks two of s.
//  Replicate  every child is the shape itself.
//  Extrude    size (s0, extent, s1).
//  Translate  t' = t + R v: t and s pass through, dL/dv_k = R[:, k] . g_t.
//  Scale      s'_k = -v_k s_k (v_k < 0), v_k (v_k > 0), 0 (v_k = 0).
//  SwapSize   s'_k = s[a_k]: dL/ds[a] = sum of g_k over the k with a_k = a.
//  IfSizeLess, If, RandomRule  discrete: the gradient passes through unchanged.
//  Generate   M[:, j] = R[:, j] s_j, M[:, 3] = t.

namespace pga {
inline namespace PGA_FRAMES_NS {

struct Grad {
  float t[3], s[3];
};

__device__ __forceinline__ void grad_zero(Grad& g) {
#pragma unroll
  for (int k = 0; k < 3; k++) g.t[k] = g.s[k] = 0.0f;
}

struct AdjArgs {
  const float* gradTerminals;  // dL/dm of terminal t: gradTerminals[t * gradStride + 0..11]
  uint32_t gradStride;         // floats, >= 12
  float* gradParams;           // numBlocks * blockStride
  uint32_t numBlocks;
  float* gradSizes;            // 3 per axiom
  float* nodeGrad;             // 6 per item: d/dt, d/ds
  uint32_t* childKey;          // per item: slot of the child with ordinal o = childKey + o
  uint32_t* pageNext;          // per item: next page of the same child, or kNoRecord
  uint32_t* slots;             // per child slot: its record (see kItemTag)
  unsigned long long* blockSums;
  unsigned long long slotCap;
};

// Dual-number evaluation of an expression program (eval_exp's postfix VM):
// every stack entry carries its value and its partials with respect to the
// shape's translation (d[0..2]) and size (d[3..5]).  Shape attributes 3, 7, 11
// are translation rows, 12..14 the size; rotation entries, the seed, the custom
// attribute, scalars and random ranges are constants here.  Comparisons and
// logic are piecewise constant.  Adds g times the partials to gx.
__device__ __noinline__ void exp_grad(const float* b, const Shape& x, float custom, float g, Grad& gx) {
  float val[PGA_MAX_EXP_LEVELS];
  float d[PGA_MAX_EXP_LEVELS][6];
  uint32_t top = 0;
  const uint32_t size = f2u(b[0]);
  for (uint32_t i = 1; i <= size && i < PGA_MAX_NUM_PARAMETER_VALUES; i++) {
    const uint32_t rbits = __float_as_uint(b[i]);
    const uint32_t kind = rbits >> 30;
    const float v = __uint_as_float(rbits << 2);
    float cv = 0.0f, cd[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (kind == 0) {
      cv = v;
    } else if (kind == 1) {
      const float hi = __fdiv_rn(fmodf(v, 4096.0f), 4095.0f);
      const float lo = __fdiv_rn(floorf(__fdiv_rn(v, 4096.0f)), 4095.0f);
      cv = rand_range(x.seed, lo, hi);
    } else if (kind == 2) {
      const uint32_t attr = f2u(roundf(v));
      cv = shape_attr(x, attr, custom);
      if (attr < 12 && (attr & 3u) == 3u) cd[attr >> 2] = 1.0f;
      if (attr >= 12 && attr < 15) cd[3 + attr - 12] = 1.0f;
    } else {
      if (top < 2) return;
      const uint32_t bi = --top, ai = --top;
      const float p1 = val[ai], p2 = val[bi];
      const uint32_t op = f2u(roundf(v));
      switch (op) {
        case 0: cv = p1 + p2; for (int q = 0; q < 6; q++) cd[q] = d[ai][q] + d[bi][q]; break;
        case 1: cv = p1 - p2; for (int q = 0; q < 6; q++) cd[q] = d[ai][q] - d[bi][q]; break;
        case 2:
          cv = p1 / p2;
          for (int q = 0; q < 6; q++) cd[q] = (d[ai][q] - cv * d[bi][q]) / p2;
          break;
        case 3: cv = p1 * p2; for (int q = 0; q < 6; q++) cd[q] = d[ai][q] * p2 + p1 * d[bi][q]; break;
        default: cv = 0.0f; break;  // comparisons and logic: zero partials
      }
    }
    if (top >= PGA_MAX_EXP_LEVELS) return;
    val[top] = cv;
    for (int q = 0; q < 6; q++) d[top][q] = cd[q];
    top++;
  }
  if (top == 0) return;
  for (int q = 0; q < 3; q++) {
    gx.t[q] += g * d[top - 1][q];
    gx.s[q] += g * d[top - 1][3 + q];
  }
}

// atomicAdd(addr, v) with the lanes of the warp that add to the same address
// summed first (shuffles over the group), so that a group makes one atomic:
// the items of one axiom, expanded side by side, add to the same few block
// gradients.
__device__ __forceinline__ void atomic_add_grouped(float* addr, float v) {
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, (unsigned long long)addr);
  if ((peers & (peers - 1u)) == 0u) {
    atomicAdd(addr, v);
    return;
  }
  float sum = 0.0f;
  for (unsigned m = peers; m != 0u; m &= m - 1u) sum += __shfl_sync(peers, v, __ffs(m) - 1);
  if ((int)(threadIdx.x & 31u) == __ffs(peers) - 1) atomicAdd(addr, sum);
}

// Gradient g of a parameter evaluated on shape x: a block value feeds the
// parameter gradient; a translation or size attribute (Shape::at 3/7/11,
// 12..14) and an expression reading them feed gx, the gradient of x (null
// where x's reads carry no gradient); every other kind is a constant of the
// grammar.
__device__ __forceinline__ void param_grad(const DeriveArgs& a, const AdjArgs& j, const DevRule& r, uint32_t k,
                                           const Shape& x, float g, Grad* gx) {
  if (g == 0.0f) return;
  const DevParam p = param_at(a, r.paramBase + k);
  if (p.type == PGA_PT_BLOCK) {
    const uint32_t slot = f2u(p.v0);
    const uint32_t b = __ldg(&a.axioms[x.axiom].block);
    if (j.gradParams != nullptr && slot < a.blockStride && b < j.numBlocks) {
#if PGA_INLINE_BLOCKS
      atomic_add_grouped(&j.gradParams[(size_t)b * a.blockStride + slot], g);
#else
      atomicAdd(&j.gradParams[(size_t)b * a.blockStride + slot], g);
#endif
    }
  } else if (p.type == PGA_PT_SHAPE_ATTR && gx != nullptr) {
    const uint32_t i = f2u(p.v0);
    if (i >= 12 && i < 15) gx->s[i - 12] += g;
    if (i < 12 && (i & 3u) == 3u) gx->t[i >> 2] += g;
  } else if (p.type == PGA_PT_EXP && gx != nullptr) {
    exp_grad(a.tab.expPool + p.aux, x, __ldg(&a.axioms[x.axiom].custom), g, *gx);
  }
}

// d(offset along the split axis) seen through the translation: R[:,a] . g_t,
// which for a signed-permutation frame is +-g_t in row perm_a.
__device__ __forceinline__ float axis_dot(const Shape& x, uint32_t ax, const float gt[3]) {
#if PGA_GENERAL_FRAMES
  // general frames: t' = t + R[:,ax] * o, so dL/do = R[:,ax] . g_t
  return frame_at(x, 0, ax) * gt[0] + frame_at(x, 1, ax) * gt[1] + frame_at(x, 2, ax) * gt[2];
#else
  const float v = pick3(gt, frame_row(x.frame, ax));
  return frame_neg(x.frame, ax) ? -v : v;
#endif
}

// Per-child terms of a Subdivide's VJP, gathered over the children of one
// work item (child_vjp) and swept back through the recurrence once
// (subdivide_sweep).
constexpr uint32_t kMaxN = PGA_MAX_NUM_PARAMETERS;
struct SubAcc {
  int last;          // highest child slot gathered; -1: none
  float gN[kMaxN];   // dL/dN_i, child i's size along the split axis
  float goI[kMaxN];  // dL/do_i, child i's offset along the split axis
};

// A Subdivide child's terms through the recurrence: dL/dN and dL/do of slot idx.
struct SubTerm {
  int idx;  // -1: none
  float gN, goI;
};

// Per-page sums for the factor and extent gradients of operators whose
// parameters do not read the shape, issued once per page (one add per factor)
// instead of once per child (the block build, PGA_INLINE_BLOCKS: the other
// builds serve tables without block parameters, whose per-child path needs
// fewer registers).  A Subdivide with at most kPureMax factors:
// W[k] = sum over the page's children of the coefficient of dN_k in dL
// (gN for the child's own slot, go / 2 there and go for every slot below it),
// Q = sum of W[k] f_k over the negative (relative) f_k.  A Repeat: the extent
// parameter's gradient.
constexpr uint32_t kPureMax = 4;
struct PageAcc {
  float W[kPureMax];
  float Q;
  float ext;
};

__device__ __forceinline__ void sub_add(SubAcc& acc, int idx, float gN, float goI) {
  if (idx < 0 || idx >= (int)kMaxN) return;
  while (acc.last < idx) {
    acc.last++;
    acc.gN[acc.last] = 0.0f;
    acc.goI[acc.last] = 0.0f;
  }
  acc.gN[idx] += gN;
  acc.goI[idx] += goI;
}

// VJP of child c of the item held in E0 (state before producing children,
// i.e. right after expander_init).  gc is the gradient of the child's state;
// the parent's gradient is accumulated into gp, except a Subdivide's terms
// through its recurrence, which are returned in st for subdivide_sweep.
__device__ __forceinline__ void child_vjp(const DeriveArgs& a, const AdjArgs& j, const Expander& E0, uint32_t c,
                                          const Grad& gc, Grad& gp, SubTerm& st, PageAcc& pa) {
  const Shape& x = E0.base;
  const DevRule& r = E0.r;
#pragma unroll
  for (int k = 0; k < 3; k++) gp.t[k] += gc.t[k];
  switch (r.op) {
    case PGA_OP_SUBDIVIDE:
    case PGA_OP_SUBDIVIDE_STATIC: {
      const bool dyn = r.op == PGA_OP_SUBDIVIDE;
      const uint32_t n = dyn ? r.nParams - 1u : r.nChildren;
      const uint32_t ax = E0.axis;
      for (uint32_t k = 0; k < 3; k++)
        if (k != ax) gp.s[k] += gc.s[k];
      const uint32_t i = min(c, n - 1u);
      const float gN = pick3(gc.s, ax), go = axis_dot(x, ax, gc.t);
      const bool scalar = (r.flags & kRuleScalar) != 0;
      if (scalar || (PGA_INLINE_BLOCKS && (r.flags & kRulePure) && n <= kPureMax)) {
        // Factors that do not read the shape: N_k = f_k (f_k > 0) or
        // scale * -f_k (f_k < 0) with scale = (S - sum of the positive f) /
        // relSum, relSum = sum of -f over the negative f, and
        // o_c = -S/2 + sum_{k<c} N_k + N_c/2.  So dN_k/dS = -f_k / relSum
        // (f_k < 0, else 0) and do_c/dS = -1/2 + sum_{k<c} dN_k/dS + dN_c/dS / 2:
        // child c's whole share of dL/dS, with nothing left for
        // subdivide_sweep.  Block factors also get their gradient, gathered
        // in pa and issued once per page (pure_factor_grads).
        float relSum = 0.0f, below = 0.0f, fc = 0.0f;
        for (uint32_t k = 0; k < n; k++) {
          const float f = scalar ? param_at(a, r.paramBase + k + 1).v0 : param(a, r, k + 1, x);
          if (f < 0.0f) {
            relSum += -f;
            if (k < i) below += -f;
          }
          if (k == i) fc = f;
        }
        float gS = -0.5f * go;
        if (relSum != 0.0f) {
          const float dN = fc < 0.0f ? -fc / relSum : 0.0f;
          gS += gN * dN + go * (below / relSum + 0.5f * dN);
        }
        gp.s[0] += (ax == 0) ? gS : 0.0f;
        gp.s[1] += (ax == 1) ? gS : 0.0f;
        gp.s[2] += (ax == 2) ? gS : 0.0f;
        if (PGA_INLINE_BLOCKS && !scalar) {
          const float own = gN + 0.5f * go;
#pragma unroll
          for (uint32_t k = 0; k < kPureMax; k++) pa.W[k] += (k == i) ? own : ((k < i) ? go : 0.0f);
          pa.Q += go * -below + own * (fc < 0.0f ? fc : 0.0f);
        }
        return;
      }
      st.idx = (int)i;
      st.gN = gN;
      st.goI = go;
      return;
    }
    case PGA_OP_REPEAT: {
      const RepeatSetup R = repeat_setup(a, r, x, false);
      const uint32_t ax = R.axis, reps = R.reps;
      const bool start = (R.flags & 2u) != 0;
      const uint32_t mode = f2u(param(a, r, 2, x));
      const float go = axis_dot(x, ax, gc.t);
      const float gsize = pick3(gc.s, ax);
      for (uint32_t k = 0; k < 3; k++)
        if (k != ax) gp.s[k] += gc.s[k];
      const bool first = (c == 0), last = (c > 0 && c + 1 >= reps), middle = !first && !last;
      float gStart = first ? (0.5f * go + gsize) : go;
      float gE2 = middle ? (go * ((float)c - 0.5f) + gsize) : (last ? go * (float)(reps - 2) : 0.0f);
      float gEnd = last ? (0.5f * go + gsize) : 0.0f;
      if (first && reps <= 1) gE2 = 0.0f;
      float gS = -0.5f * go, gE = 0.0f;
      const float S = pick3(x.s, ax);
      const float ext = param(a, r, 1, x);
      const float E = ext < 0.0f ? S * fabsf(ext) : ext;
      if (mode == 2u) {
        if (reps > 0) gS += (gStart + gE2 + gEnd) / (float)reps;
      } else {
        const float ge1 = start ? gStart : gEnd;
        gE += (start ? gEnd : gStart) + gE2;
        const float rest = fmodf(S, E);
        if (rest == 0.0f) {
          gE += ge1;
        } else {
          gS += ge1;
          gE += -truncf(S / E) * ge1;
        }
      }
#if PGA_INLINE_BLOCKS
      if (ext < 0.0f) {
        gS += gE * fabsf(ext);
        pa.ext += gE * (-S);
      } else {
        pa.ext += gE;
      }
#else
      if (ext < 0.0f) {
        gS += gE * fabsf(ext);
        param_grad(a, j, r, 1, x, gE * (-S), &gp);
      } else {
        param_grad(a, j, r, 1, x, gE, &gp);
      }
#endif
      gp.s[0] += (ax == 0) ? gS : 0.0f;
      gp.s[1] += (ax == 1) ? gS : 0.0f;
      gp.s[2] += (ax == 2) ? gS : 0.0f;
      return;
    }
    case PGA_OP_COMPONENT_SPLIT: {
      // face c: translation axis k and sign, face size (x, y) from parent components.
      uint32_t k, m0, m1;
      float sgn;
      switch (c) {
        case 0: k = 2; sgn = -1.0f; m0 = 0; m1 = 1; break;
        case 1: k = 2; sgn = 1.0f; m0 = 0; m1 = 1; break;
        case 2: k = 0; sgn = -1.0f; m0 = 2; m1 = 1; break;
        case 3: k = 0; sgn = 1.0f; m0 = 2; m1 = 1; break;
        case 4: k = 1; sgn = -1.0f; m0 = 0; m1 = 2; break;
        default: k = 1; sgn = 1.0f; m0 = 0; m1 = 2; break;
      }
      const float go = axis_dot(x, k, gc.t);
      float add[3] = {0.0f, 0.0f, 0.0f};
      add[k] += sgn * 0.5f * go;
      add[m0] += gc.s[0];
      add[m1] += gc.s[1];
#pragma unroll
      for (int q = 0; q < 3; q++) gp.s[q] += add[q];
      return;
    }
    case PGA_OP_REPLICATE:
#pragma unroll
      for (int q = 0; q < 3; q++) gp.s[q] += gc.s[q];
      return;
    default:
      return;
  }
}

// The reverse pass of a Subdivide over the terms gathered in acc, into gp.
__device__ void subdivide_sweep(const DeriveArgs& a, const AdjArgs& j, const Expander& E0, SubAcc& acc, Grad& gp) {
  if (acc.last < 0) return;
  const Shape& x = E0.base;
  const DevRule& r = E0.r;
  const bool dyn = r.op == PGA_OP_SUBDIVIDE;
  const uint32_t n = dyn ? r.nParams - 1u : r.nChildren;
  const uint32_t ax = E0.axis;
  // Reverse pass over the recurrence that produced the children:
  //   offset_0 = -S/2;  N_i = size(f_i, scale);  o_i = offset_i + N_i/2;
  //   offset_{i+1} = offset_i + N_i;  child c: size N_c, translation t + R_a o_c.
  // Factor f_i is read on the base shape (static form, i = 0, or a rule
  // whose factors do not read the shape) or, for a dynamic Subdivide, on the
  // symbol as child i - 1 left it in place: size N_{i-1} along a and
  // translation t + R_a o_{i-1}; its gradient then flows to N_{i-1},
  // o_{i-1} and the base's other sizes and translation.  The scale uses
  // the factors read from the base shape.
  float fv[kMaxN], Nv[kMaxN], ov[kMaxN];
  const uint32_t last = (uint32_t)acc.last;
  Expander W = E0;
  for (uint32_t i = 0; i <= last && i < kMaxN; i++) {
    const float f = dyn ? dyn_factor(a, W, i) : param(a, r, i + 1, x);
    const float sz = subdivide_size(f, W.scale);
    fv[i] = f;
    Nv[i] = sz;
    ov[i] = __fadd_rn(W.offset, __fmul_rn(sz, 0.5f));
    W.prevOff = ov[i];
    W.prevSize = sz;
    W.offset = __fadd_rn(W.offset, sz);
  }
  const bool readsUpdated = dyn && !(r.flags & kRulePure);
  float gS = 0.0f, gscale = 0.0f, gOffNext = 0.0f;
  for (int i = (int)last; i >= 0; i--) {
    // o_i = offset_i + N_i/2 and offset_{i+1} = offset_i + N_i
    const float gOff = gOffNext + acc.goI[i];
    acc.gN[i] += gOffNext + 0.5f * acc.goI[i];
    gOffNext = gOff;
    const float f = fv[i];
    if (!dyn && f == 0.0f) continue;  // a skipped static slot
    float gf = 0.0f;
    if (f > 0.0f) {
      gf = acc.gN[i];
    } else if (f < 0.0f) {
      gf = acc.gN[i] * (-E0.scale);
      gscale += acc.gN[i] * (-f);
    }
    if (gf == 0.0f) continue;
    if (!readsUpdated || i == 0) {
      param_grad(a, j, r, i + 1, x, gf, &gp);
    } else {
      Shape cur = x;
      put3(cur.s, ax, Nv[i - 1]);
      translate_ref(cur, x, E0.axisRef, ov[i - 1]);
      cur.seed = seed_of(a, x.seed, (uint32_t)i - 1u);
      Grad gst;
      grad_zero(gst);
      param_grad(a, j, r, i + 1, cur, gf, &gst);
      acc.gN[i - 1] += pick3(gst.s, ax);
      for (uint32_t k = 0; k < 3; k++)
        if (k != ax) gp.s[k] += gst.s[k];
#pragma unroll
      for (int q = 0; q < 3; q++) gp.t[q] += gst.t[q];
      acc.goI[i - 1] += axis_dot(x, ax, gst.t);
    }
  }
  gS += -0.5f * gOffNext;  // offset_0 = -S/2
  if (gscale != 0.0f) {
    float relSum = 0.0f;
    for (uint32_t i = 0; i < n; i++) {
      const float f = param(a, r, i + 1, x);
      if (f < 0.0f) relSum += -f;
    }
    if (relSum != 0.0f) {
      // scale = (S - sum_{f>0} f) / sum_{f<0} -f
      gS += gscale / relSum;
      const float gA = -gscale / relSum, gR = gscale * E0.scale / relSum;
      for (uint32_t i = 0; i < n; i++) {
        const float f = param(a, r, i + 1, x);
        if (f > 0.0f) param_grad(a, j, r, i + 1, x, gA, &gp);
        if (f < 0.0f) param_grad(a, j, r, i + 1, x, gR, &gp);
      }
    }
  }
  gp.s[0] += (ax == 0) ? gS : 0.0f;
  gp.s[1] += (ax == 1) ? gS : 0.0f;
  gp.s[2] += (ax == 2) ? gS : 0.0f;
}

// The 1 -> 1 chain a created shape runs through before it becomes a record
// (a terminal, a queued work item, or nothing): IfSizeLess, If and RandomRule
// pick a branch and pass the gradient through unchanged; the smooth steps
// (Extrude, Translate, Scale, SwapSize) are recorded so that the reverse pass
// can undo them.  A chain with more than kChainSteps of them has no adjoint
// (PGA_ERR_NO_TAPE).
// The share of a wide level that the adjoint hands out dynamically: 1 / this
// (1: all of it; measured on the 65,536-axiom step, sizes / all parameters:
// a quarter 22 / 57-66 ms, half 20.3 / 40-46 ms, all 19.3 / 35 ms).
#ifndef PGA_ADJOINT_DYNAMIC_SHARE
#define PGA_ADJOINT_DYNAMIC_SHARE 1
#endif

constexpr int kChainSteps = 8;
struct Chain {
  uint32_t n;                   // smooth steps
  int32_t entry[kChainSteps];   // rule of each step
  Shape before[kChainSteps];    // state entering each step
};

enum ChainEnd : int { kEndFail = -1, kEndTerminal = 0, kEndItem = 1, kEndDiscard = 2 };

// Replays the chain from x, the shape as its creator produced it, to its end
// state yEnd (the record's state; its path hash is not kept up to date, the
// reverse pass has no use for it); returns how it ends.
__device__ int replay_chain(const DeriveArgs& a, Shape x, Chain& ch, Shape& yEnd) {
  ch.n = 0;
  for (int step = 0; step < kMaxChain; step++) {
    if (x.entry < 0 || (uint32_t)x.entry >= a.tab.numEntries) return kEndFail;
    const DevRule r = rule_at(a, (uint32_t)x.entry);
    if (r.op == PGA_OP_IF_SIZE_LESS) {
      uint32_t axis;
      if (!axis_param(a, r, x, axis)) return kEndFail;
      const float size = param(a, r, 1, x);
      const uint32_t branch = (pick3(x.s, axis) < size) ? 0u : 1u;
      x.entry = succ_at(a, r.succBase + branch);
      continue;
    }
    if (r.op == PGA_OP_RANDOM_RULE || r.op == PGA_OP_RANDOM_RULE_STATIC) {
      const int pick = random_pick(a, r, x);
      if (pick < 0) return kEndFail;
      const int32_t nxt = succ_at(a, r.succBase + (uint32_t)pick);
      x.entry = nxt;
      continue;
    }
    if (r.op == PGA_OP_IF) {
      const uint32_t branch = (param(a, r, 0, x) != 0.0f) ? 0u : 1u;
      x.entry = succ_at(a, r.succBase + branch);
      continue;
    }
#if PGA_GENERAL_FRAMES
    if (r.op == PGA_OP_ROTATE) {
      // model * rotateXYZ of scalar angles (built at engine creation): the
      // frame turns, translation and size pass through, and no continuous
      // input reaches the rotation, so the gradient passes through unchanged
      frame_rotate(x, a.tab.expPool + param_at(a, r.paramBase).aux);
      x.entry = succ_at(a, r.succBase);
      continue;
    }
#endif
    if (r.op == PGA_OP_TRANSLATE || r.op == PGA_OP_SCALE || r.op == PGA_OP_SWAP_SIZE) {
      if (ch.n >= kChainSteps) return kEndFail;
      ch.entry[ch.n] = x.entry;
      ch.before[ch.n] = x;
      ch.n++;
      if (r.op == PGA_OP_TRANSLATE)
        apply_translate(a, r, x);
      else if (r.op == PGA_OP_SCALE)
        apply_scale(a, r, x);
      else if (!swap_size(a, r, x))
        return kEndFail;
      x.entry = succ_at(a, r.succBase);
      continue;
    }
    if (r.op == PGA_OP_EXTRUDE) {
      if (ch.n >= kChainSteps) return kEndFail;
      ch.entry[ch.n] = x.entry;
      ch.before[ch.n] = x;
      ch.n++;
      const float extent = param(a, r, 1, x);
      frame_set2(x, x, 1, 2, 0, 2, 1, 1);  // model * [x, z, -y] columns, as the forward
      x.s[2] = x.s[1];
      x.s[1] = extent;
      x.seed = seed_of(a, x.seed, 0u);
      x.kind = PGA_SHAPE_BOX;
      const int32_t nxt = succ_at(a, r.succBase);
      x.entry = nxt;
      continue;
    }
    yEnd = x;
    if (r.op == PGA_OP_GENERATE) return kEndTerminal;
    return r.op == PGA_OP_DISCARD ? kEndDiscard : kEndItem;
  }
  return kEndFail;
}

// Undoes the smooth steps of ch, last first: g, the gradient of the chain's
// end state, becomes that of the state it started from.  Parameter gradients
// go to j.gradParams.
__device__ void chain_vjp(const DeriveArgs& a, const AdjArgs& j, const Chain& ch, Grad& g) {
  for (int k = (int)ch.n - 1; k >= 0; k--) {
    const Shape& xb = ch.before[k];
    const DevRule r = rule_at(a, (uint32_t)ch.entry[k]);
    Grad gb;
#pragma unroll
    for (int q = 0; q < 3; q++) gb.t[q] = g.t[q];
    if (r.op == PGA_OP_TRANSLATE) {
#pragma unroll
      for (int q = 0; q < 3; q++) gb.s[q] = g.s[q];
      for (uint32_t q = 0; q < 3; q++) param_grad(a, j, r, q, xb, axis_dot(xb, q, g.t), &gb);
    } else if (r.op == PGA_OP_SCALE) {
      float v[3], dv[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        v[q] = param(a, r, (uint32_t)q, xb);
        gb.s[q] = (v[q] < 0.0f) ? -v[q] * g.s[q] : 0.0f;
        dv[q] = (v[q] < 0.0f) ? -xb.s[q] : (v[q] > 0.0f ? 1.0f : 0.0f);
      }
      for (uint32_t q = 0; q < 3; q++) param_grad(a, j, r, q, xb, g.s[q] * dv[q], &gb);
    } else if (r.op == PGA_OP_SWAP_SIZE) {
      // after[k] = before[axis_k]: each component's gradient goes back to the axis it was read from
      const uint32_t a0 = f2u(param(a, r, 0, xb)), a1 = f2u(param(a, r, 1, xb)), a2 = f2u(param(a, r, 2, xb));
#pragma unroll
      for (uint32_t q = 0; q < 3; q++)
        gb.s[q] = (a0 == q ? g.s[0] : 0.0f) + (a1 == q ? g.s[1] : 0.0f) + (a2 == q ? g.s[2] : 0.0f);
    } else {  // Extrude: after = (s0, extent, s1)
      gb.s[0] = g.s[0];
      gb.s[1] = g.s[2];
      gb.s[2] = 0.0f;
      param_grad(a, j, r, 1, xb, g.s[1], &gb);
    }
    g = gb;
  }
}

// dL/d(state) of a Generate rule's shape y from dL/dM of its terminal t:
// M[:, k] = R[:, k] s_k and M[:, 3] = t.
__device__ __forceinline__ Grad terminal_grad(const AdjArgs& j, unsigned long long t, const Shape& y) {
  const float* gm = j.gradTerminals + t * j.gradStride;
  Grad g;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    g.t[q] = __ldg(gm + q * 4 + 3);
#if PGA_GENERAL_FRAMES
    // M[i][q] = R[i][q] s_q: dL/ds_q = sum_i dL/dM[i][q] R[i][q]
    g.s[q] = __ldg(gm + q) * frame_at(y, 0, q) + __ldg(gm + 4 + q) * frame_at(y, 1, q) +
             __ldg(gm + 8 + q) * frame_at(y, 2, q);
#else
    const uint32_t row = frame_row(y.frame, q);
    const float v = __ldg(gm + row * 4 + q);
    g.s[q] = frame_neg(y.frame, q) ? -v : v;
#endif
  }
  return g;
}

// A record created from axiom ax's root shape (a terminal t, or a work item
// whose gradient is g): back through the root's chain into the axiom's size
// gradient.  An axiom has few such records (one terminal, or the pages of
// one item), so they add atomically; out of line, as the rare path it is.
__device__ __noinline__ void push_to_axiom(const DeriveArgs& a, const AdjArgs& j, uint32_t ax, bool terminal,
                                           unsigned long long t, Grad g) {
  Shape y0, yEnd;
  axiom_shape(a, ax, y0);
  Chain ch;
  if (replay_chain(a, y0, ch, yEnd) != (terminal ? kEndTerminal : kEndItem)) {
    raise_error(a.st, PGA_ERR_NO_TAPE, (int)ax);
    return;
  }
  if (terminal) g = terminal_grad(j, t, yEnd);
  chain_vjp(a, j, ch, g);
  if (j.gradSizes != nullptr)
    for (int q = 0; q < 3; q++)
      if (g.s[q] != 0.0f) atomicAdd(&j.gradSizes[(size_t)ax * 3 + q], g.s[q]);
}

// The slot map.  Work item i (one page of a queued shape: its children
// [c0, c1)) owns the slots [base_i, base_i + c1 - c0), base_i an exclusive
// scan of the pages' child counts; childKey_i = base_i - c0 - (1 for Repeat,
// whose child c has ordinal c + 1), so the child with tape link
// (i, ordinal) sits at childKey_i + ordinal.  A slot holds the terminal the
// child became, or the first of the pages it was queued as (kItemTag | page,
// the others linked through pageNext), or kNoRecord (discarded).
constexpr uint32_t kNoRecord = 0xFFFFFFFFu;
constexpr uint32_t kItemTag = 0x80000000u;

__device__ __forceinline__ uint32_t page_children(const uint4& ext) {
  return ext.x == kEmptyItem ? 0u : ext.y - ext.x;
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Slots read ahead per work item (a work item has max(subItem, narrowSubItem)
// children at most, 8 by default).
constexpr uint32_t kPrefetch = 8;

// Gradient of a child queued as the pages in the list starting at v: the sum
// of their gradients (each page's covers its own children).
__device__ __forceinline__ Grad pages_grad(const AdjArgs& j, uint32_t v, unsigned long long nodes) {
  Grad g;
  grad_zero(g);
  uint32_t k = v & ~kItemTag;
  for (unsigned long long guard = 0; k != kNoRecord && k < nodes && guard < nodes; guard++) {
    const float* src = j.nodeGrad + (size_t)k * 6;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      g.t[q] += __ldcg(src + q);
      g.s[q] += __ldcg(src + 3 + q);
    }
    k = __ldcg(j.pageNext + k);
  }
  return g;
}

// The page's gathered parameter gradients (PageAcc): a Repeat's extent, and
// the factors of a Subdivide whose factors do not read the shape (at most
// kPureMax): dL/df_j = W_j + Q / relSum for f_j > 0 and
// -(W_j + Q / relSum) * scale for f_j < 0 (the size terms through N_j and,
// via scale, through every relative N_k).
__device__ __forceinline__ void page_param_grads(const DeriveArgs& a, const AdjArgs& j, const Expander& E,
                                                 const PageAcc& pa, Grad& gp) {
  const DevRule& r = E.r;
  const Shape& x = E.base;
  if (r.op == PGA_OP_REPEAT) {
    param_grad(a, j, r, 1, x, pa.ext, &gp);
    return;
  }
  if ((r.op != PGA_OP_SUBDIVIDE && r.op != PGA_OP_SUBDIVIDE_STATIC) || (r.flags & kRuleScalar) ||
      !(r.flags & kRulePure))
    return;
  const uint32_t n = r.op == PGA_OP_SUBDIVIDE ? r.nParams - 1u : r.nChildren;
  if (n > kPureMax) return;
  float f[kPureMax], relSum = 0.0f;
#pragma unroll
  for (uint32_t k = 0; k < kPureMax; k++) {
    f[k] = k < n ? param(a, r, k + 1, x) : 0.0f;
    relSum += f[k] < 0.0f ? -f[k] : 0.0f;
  }
  const float q = relSum != 0.0f ? pa.Q / relSum : 0.0f;
#pragma unroll
  for (uint32_t k = 0; k < kPureMax; k++) {
    if (k >= n) break;
    const float g = f[k] > 0.0f ? pa.W[k] + q : (f[k] < 0.0f ? -(pa.W[k] + q) * E.scale : 0.0f);
    param_grad(a, j, r, k + 1, x, g, &gp);
  }
}

// Reverse step of work item i: its children in order -- each one's gradient
// read through the slot map (a terminal's dL/dM, or the sum over the pages it
// was queued as) and pushed back through its chain and the operator that
// created it -- summed into the item's gradient, which is stored (or, for an
// axiom's root item, pushed into the axiom's sizes).
__device__ void adj_page(const DeriveArgs& a, const AdjArgs& j, unsigned long long i, unsigned long long nodes) {
  Expander E;
  uint4 ext;
  load_node(a, i, E.base, ext);
  if (ext.x == kEmptyItem) return;
  const int32_t e = E.base.entry;
  if (e < 0 || (uint32_t)e >= a.tab.numEntries) {
    raise_error(a.st, PGA_ERR_NO_TAPE, (int)i);
    return;
  }
  E.r = rule_at(a, (uint32_t)e);
  E.base.kind = E.r.shape;
  const uint32_t all = expander_init(a, E);
  const uint32_t c0 = ext.x, c1 = min(ext.y, all);
  const uint32_t key = __ldcg(j.childKey + i);
  {
    // Start the loads of the children's slots and of the gradients they
    // point to, so that their latencies overlap instead of adding up child
    // after child below (a child's slot is key + c + 1 for Repeat, else key + c).
    const uint32_t rep = E.r.op == PGA_OP_REPEAT ? 1u : 0u;
    uint32_t sv[kPrefetch];
#pragma unroll
    for (uint32_t q = 0; q < kPrefetch; q++)
      sv[q] = (c0 + q < c1) ? __ldcg(j.slots + (uint32_t)(key + c0 + q + rep)) : kNoRecord;
#pragma unroll
    for (uint32_t q = 0; q < kPrefetch; q++) {
      if (sv[q] == kNoRecord) continue;
      if (sv[q] & kItemTag) {
        prefetch_l2(j.nodeGrad + (size_t)(sv[q] & ~kItemTag) * 6);
      } else {
        const float* gm = j.gradTerminals + (size_t)sv[q] * j.gradStride;
        prefetch_l2(gm);
        prefetch_l2(gm + 11);
      }
    }
  }
  Grad gp;
  grad_zero(gp);
  SubAcc acc;
  acc.last = -1;
  PageAcc pa;
#pragma unroll
  for (uint32_t k = 0; k < kPureMax; k++) pa.W[k] = 0.0f;
  pa.Q = 0.0f;
  pa.ext = 0.0f;
  Expander W = E;
  if (c0 < c1) expander_skip(a, W, c0);
  for (uint32_t c = c0; c < c1; c++) {
    Shape y0, yEnd;
    uint32_t ord;
    if (!expander_child<1, false>(a, W, c, y0, ord)) continue;
    const uint32_t v = __ldcg(j.slots + (uint32_t)(key + ord));
    if (v == kNoRecord) continue;  // discarded
    Chain ch;
    const int end = replay_chain(a, y0, ch, yEnd);
    Grad g;
    if (end == kEndTerminal && !(v & kItemTag)) {
      g = terminal_grad(j, v, yEnd);
    } else if (end == kEndItem && (v & kItemTag)) {
      g = pages_grad(j, v, nodes);
    } else {
      raise_error(a.st, PGA_ERR_NO_TAPE, (int)i);
      return;
    }
    chain_vjp(a, j, ch, g);
    SubTerm st;
    st.idx = -1;
    child_vjp(a, j, E, c, g, gp, st, pa);
    sub_add(acc, st.idx, st.gN, st.goI);
  }
#if PGA_INLINE_BLOCKS
  page_param_grads(a, j, E, pa, gp);
#endif
  subdivide_sweep(a, j, E, acc, gp);
  if (ext.z & kAxiomLink) {
    push_to_axiom(a, j, ext.z & ~kAxiomLink, false, 0, gp);
    return;
  }
  float* dst = j.nodeGrad + (size_t)i * 6;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    __stcg(dst + q, gp.t[q]);
    __stcg(dst + 3 + q, gp.s[q]);
  }
}

// Block-wide exclusive scan of one value per thread; total receives the sum.
__device__ __forceinline__ unsigned long long block_excl_scan(uint32_t v, unsigned long long& total) {
  __shared__ unsigned long long warpSum[kWarps];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  uint32_t wt;
  const uint32_t pre = warp_excl_scan(v, wt);
  if (lane == 0) warpSum[warp] = wt;
  __syncthreads();
  unsigned long long before = 0, all = 0;
  for (int w = 0; w < kWarps; w++) {
    const unsigned long long x = warpSum[w];
    before += (w < (int)warp) ? x : 0ull;
    all += x;
  }
  __syncthreads();
  total = all;
  return before + pre;
}

__device__ __forceinline__ unsigned long long block_sum(unsigned long long v) {
  __shared__ unsigned long long part[kWarps];
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(kFull, v, d);
  if ((threadIdx.x & 31u) == 0) part[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long s = 0;
  for (int w = 0; w < kWarps; w++) s += part[w];
  __syncthreads();
  return s;
}

// The whole reverse sweep in one cooperative launch, with a bounded grid
// barrier after each phase:
//   1. zero the outputs; each block sums the child counts of its contiguous
//      chunk of work items;
//   2. each block scans its chunk into child keys and marks its slots empty;
//   3. every terminal and work item enters its slot (a terminal of an axiom's
//      root goes straight to the axiom's sizes);
//   4. the levels from the deepest up, one adj_page per work item.
// The level bounds, the item and the terminal counts are the forward launch's
// final state, read on the device, so no host round trip is needed.  A failed
// or overflowed forward pass leaves the gradients zero (the engine report
// keeps the forward's status; a tape too short for the terminals or a slot
// map larger than its buffer raises PGA_ERR_NO_TAPE).
// Two launch shapes of the same pass.  k_adjoint keeps the compiler's
// register choice (2 blocks of 256 per SM; the block build pins 2 blocks: left
// free, its choice there came out at 80 registers with spills).
// k_adjoint_wide (frame-code builds) runs 3 blocks per SM (80 registers, ~300
// B of spills; the block build 4 blocks, 64 registers): with the level's pages handed out on demand the extra warps
// hide more of the scattered reads on large tapes (65,536-axiom step: sizes
// 19.2 -> 18.2 ms, all parameters 35 -> 32 ms), while on small ones the
// spills and the larger grid's barriers cost more (1,024 facades: forward +
// adjoint 0.264 -> 0.302 ms).  Engines choose by terminal capacity
// (kWideAdjointTerminals).  PGA_ADJOINT_MIN_BLOCKS overrides k_adjoint's shape.
#if defined(PGA_ADJOINT_MIN_BLOCKS)
#define PGA_ADJOINT_BOUNDS __launch_bounds__(kThreads, PGA_ADJOINT_MIN_BLOCKS)
#elif PGA_INLINE_BLOCKS
#define PGA_ADJOINT_BOUNDS __launch_bounds__(kThreads, 2)
#else
#define PGA_ADJOINT_BOUNDS __launch_bounds__(kThreads)
#endif
__device__ __forceinline__ void adjoint_pass(const DeriveArgs& a, const AdjArgs& j, unsigned long long numParamFloats,
                                             uint32_t numAxioms) {
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  setup_block(a, sm);
  volatile DevState* vs = a.st;
  // Fixed by the forward launch; nothing below changes them before the first barrier.
  const unsigned long long nodes = min((unsigned long long)vs->nodeNext, a.nodeCap);
  const unsigned long long nTerm = vs->termCount;
  const uint32_t levels = vs->levels;
  const bool ok = vs->status == 0 && nTerm <= a.cap && nTerm <= a.termLinkCap && nTerm < kItemTag;
  const unsigned long long tid = (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  const unsigned long long stride = (unsigned long long)gridDim.x * kThreads;
  if (j.gradParams)
    for (unsigned long long k = tid; k < numParamFloats; k += stride) j.gradParams[k] = 0.0f;
  if (j.gradSizes)
    for (unsigned long long k = tid; k < (unsigned long long)numAxioms * 3; k += stride) j.gradSizes[k] = 0.0f;
  // Each block owns a contiguous chunk of the work items, each thread a
  // contiguous run of its block's chunk; loads go kUnroll at a time.
  constexpr int kUnroll = 4;
  const unsigned long long chunk = (nodes + gridDim.x - 1) / gridDim.x;
  const unsigned long long lo = min((unsigned long long)blockIdx.x * chunk, nodes), hi = min(lo + chunk, nodes);
  const unsigned long long run = (hi - lo + kThreads - 1) / kThreads;
  const unsigned long long tlo = min(lo + threadIdx.x * run, hi), thi = min(tlo + run, hi);
  uint32_t mine = 0;  // a work item has at most 64 children
  for (unsigned long long i = tlo; i < thi; i += kUnroll) {
    uint4 ext[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++)
      ext[u] = i + u < thi ? __ldcg(reinterpret_cast<const uint4*>(a.nodes + i + u) + 3)
                           : make_uint4(kEmptyItem, 0u, 0u, 0u);
#pragma unroll
    for (int u = 0; u < kUnroll; u++) mine += page_children(ext[u]);
  }
  const unsigned long long blockTotal = block_sum(mine);
  if (threadIdx.x == 0) j.blockSums[blockIdx.x] = blockTotal;
  if (!grid_barrier(a, [] {})) return;
  if (!ok) {
    if (tid == 0 && vs->status == 0) raise_error(a.st, PGA_ERR_NO_TAPE, -1);
    return;
  }
  unsigned long long base = 0, total = 0;
  for (uint32_t b = threadIdx.x; b < gridDim.x; b += kThreads) {
    const unsigned long long x = __ldcg(j.blockSums + b);
    base += (b < blockIdx.x) ? x : 0ull;
    total += x;
  }
  base = block_sum(base);
  total = block_sum(total);
  if (total > j.slotCap) {  // every block sees the same total and returns here
    if (tid == 0) raise_error(a.st, PGA_ERR_NO_TAPE, -2);
    return;
  }
  for (unsigned long long k = tid; k < total; k += stride) j.slots[k] = kNoRecord;
  {
    unsigned long long ignored;
    unsigned long long first = base + block_excl_scan(mine, ignored);
    for (unsigned long long i = tlo; i < thi; i += kUnroll) {
      uint4 m[kUnroll], ext[kUnroll];
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        const uint4* rec = reinterpret_cast<const uint4*>(a.nodes + min(i + u, thi - 1));
        m[u] = __ldcg(rec + 2);
        ext[u] = __ldcg(rec + 3);
      }
#pragma unroll
      for (int u = 0; u < kUnroll; u++) {
        if (i + u >= thi) break;
        const uint32_t cnt = page_children(ext[u]);
        uint32_t key = 0;
        if (cnt) {
          const int32_t e = (int32_t)m[u].x;
          const bool rep = e >= 0 && (uint32_t)e < a.tab.numEntries && rule_at(a, (uint32_t)e).op == PGA_OP_REPEAT;
          key = (uint32_t)0u - ext[u].x - (rep ? 1u : 0u);
        }
        j.childKey[i + u] = (uint32_t)first + key;
        first += cnt;
      }
    }
  }
  if (!grid_barrier(a, [] {})) return;
  for (unsigned long long t0 = tid; t0 < nTerm; t0 += stride * kUnroll) {
    uint2 link[kUnroll];
    uint32_t key[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const unsigned long long t = t0 + u * stride;
      link[u] = t < nTerm ? __ldg(a.termLinks + t) : make_uint2(kAxiomLink, 0u);
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++)
      key[u] = (!(link[u].x & kAxiomLink) && link[u].x < nodes) ? __ldcg(j.childKey + link[u].x) : 0u;
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const unsigned long long t = t0 + u * stride;
      if (t >= nTerm) break;
      if (link[u].x & kAxiomLink) {
        Grad none;
        grad_zero(none);
        push_to_axiom(a, j, link[u].x & ~kAxiomLink, true, t, none);
      } else if (link[u].x < nodes) {
        j.slots[(uint32_t)(key[u] + link[u].y)] = (uint32_t)t;
      }
    }
  }
  for (unsigned long long i0 = tid; i0 < nodes; i0 += stride * kUnroll) {
    uint4 ext[kUnroll];
    uint32_t key[kUnroll];
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const unsigned long long i = i0 + u * stride;
      ext[u] = i < nodes ? __ldcg(reinterpret_cast<const uint4*>(a.nodes + i) + 3) : make_uint4(kEmptyItem, 0u, 0u, 0u);
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      const bool take = ext[u].x != kEmptyItem && !(ext[u].z & kAxiomLink) && ext[u].z < nodes;
      ext[u].x = take ? 0u : kEmptyItem;
      key[u] = take ? __ldcg(j.childKey + ext[u].z) : 0u;
    }
#pragma unroll
    for (int u = 0; u < kUnroll; u++) {
      if (ext[u].x == kEmptyItem) continue;
      const unsigned long long i = i0 + u * stride;
      const uint32_t head = atomicExch(j.slots + (uint32_t)(key[u] + ext[u].w), kItemTag | (uint32_t)i);
      j.pageNext[i] = head == kNoRecord ? kNoRecord : (head & ~kItemTag);
    }
  }
  // The levels, last first.  A level of at least four rounds of the grid
  // leaves its last 1 / PGA_ADJOINT_DYNAMIC_SHARE (at least two rounds) to
  // warps that take 32 items at a time from DevState::cursor, reset at each
  // barrier: pages differ widely in cost, and the gradients are sums of
  // atomics whose order was never fixed, so the order of the pages changes
  // nothing a caller sees.
  if (!grid_barrier(a, [&] { a.st->cursor = 0ull; })) return;
  for (int L = (int)levels; L >= 0; L--) {
    const unsigned long long lv = a.levelStart[L], hv = min(a.levelStart[L + 1], nodes);
    if (lv >= hv) continue;  // every block reads the same bounds, so all skip the barrier alike
    unsigned long long dynLo = hv;
    if (hv - lv >= 4 * stride) {
      const unsigned long long n = hv - lv;
      dynLo = lv + ((n - max(n / PGA_ADJOINT_DYNAMIC_SHARE, 2 * stride)) / stride) * stride;
    }
    // one call site of adj_page for both orders
    for (unsigned long long i = lv + tid;; i += stride) {
      if (i >= dynLo) {
        if (dynLo >= hv) break;
        unsigned long long c = 0;
        if ((threadIdx.x & 31u) == 0) c = atomicAdd(&a.st->cursor, 32ull);
        c = dynLo + __shfl_sync(kFull, c, 0);
        if (c >= hv) break;
        i = c + (threadIdx.x & 31u);  // the loop step never lands below dynLo again
        if (i >= hv) continue;        // this lane has no item in the last chunk
      } else if (i + stride < dynLo) {  // the next item's record and key, ahead of its turn
        prefetch_l2(a.nodes + i + stride);
        prefetch_l2(j.childKey + i + stride);
      }
      adj_page(a, j, i, nodes);
    }
    if (!grid_barrier(a, [&] { a.st->cursor = 0ull; })) return;
  }
}

__global__ void PGA_ADJOINT_BOUNDS k_adjoint(DeriveArgs a, AdjArgs j, unsigned long long numParamFloats,
                                             uint32_t numAxioms) {
  adjoint_pass(a, j, numParamFloats, numAxioms);
}

#if !PGA_GENERAL_FRAMES
#ifndef PGA_ADJOINT_WIDE_BLOCKS
#if PGA_INLINE_BLOCKS
#define PGA_ADJOINT_WIDE_BLOCKS 4  // 64 registers: all parameters 33 -> 31 ms on the 65,536-axiom step
#else
#define PGA_ADJOINT_WIDE_BLOCKS 3  // at 4 the sizes step's adjoint lost 3%
#endif
#endif
__global__ void __launch_bounds__(kThreads, PGA_ADJOINT_WIDE_BLOCKS) k_adjoint_wide(DeriveArgs a, AdjArgs j,
                                                              unsigned long long numParamFloats, uint32_t numAxioms) {
  adjoint_pass(a, j, numParamFloats, numAxioms);
}
#endif

// This build's adjoint kernels, for the host code (the general-frame build
// has one shape).
inline const void* adjoint_kernel() { return (const void*)k_adjoint; }
#if PGA_GENERAL_FRAMES
inline const void* adjoint_kernel_wide() { return (const void*)k_adjoint; }
#else
inline const void* adjoint_kernel_wide() { return (const void*)k_adjoint_wide; }
#endif

}  // inline namespace PGA_FRAMES_NS
}  // namespace pga

#ifndef PGA_ADJOINT_DEVICE_ONLY
extern "C" PgaStatus pga_adjoint_strided(PgaEngine* e, const float* dGradTerminals, uint32_t gradStride,
                                         float* dGradParams, uint32_t numBlocks, float* dGradAxiomSizes,
                                         void* stream) {
  using namespace pga;
  if (!e || !dGradTerminals) {
    set_error("pga_adjoint: null engine or gradient");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (gradStride < 12) {
    set_error("pga_adjoint_strided: gradStride must be at least 12 floats");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (!e->cfg.recordTape || !e->lastWasBatched || !e->dTermLinks || !e->lastOut || !e->kernels.adjoint) {
    set_error("pga_adjoint: the last derivation was not a pga_derive on an engine created with recordTape = 1");
    return PGA_ERR_NO_TAPE;
  }
  if (e->adjointBlocks == 0) {
    // One cooperative launch: as many blocks as can be resident with the
    // engine's dynamic shared memory.
    PGA_CUDA_TRY(cudaFuncSetAttribute(e->kernels.adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smemBytes));
    int perSM = 0;
    PGA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, e->kernels.adjoint, kThreads, e->smemBytes));
    if (perSM < 1) {
      set_error("pga_adjoint: the adjoint kernel does not fit on an SM");
      return PGA_ERR_CUDA;
    }
    e->adjointBlocks = (int)std::min<uint32_t>((uint32_t)(perSM * e->numSMs), kMaxAdjointBlocks);
  }
  DeriveArgs a = make_args(e, e->lastAxioms, e->lastNumAxioms, e->lastBlocks, e->lastOut, e->lastCap, nullptr);
  AdjArgs j;
  j.gradTerminals = dGradTerminals;
  j.gradStride = gradStride;
  j.gradParams = dGradParams;
  j.numBlocks = numBlocks;
  j.gradSizes = dGradAxiomSizes;
  j.nodeGrad = e->dNodeGrad;
  j.childKey = e->dChildKey;
  j.pageNext = e->dPageNext;
  j.slots = e->dSlots;
  j.blockSums = e->dBlockSums;
  j.slotCap = e->slotCap;
  unsigned long long numParamFloats = (unsigned long long)numBlocks * e->cfg.blockStride;
  uint32_t numAxioms = e->lastNumAxioms;
  void* args[] = {&a, &j, &numParamFloats, &numAxioms};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)e->adjointBlocks);
  cfg.blockDim = dim3((unsigned)kThreads);
  cfg.dynamicSmemBytes = e->smemBytes;
  cfg.stream = (cudaStream_t)stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  PGA_CUDA_TRY(cudaLaunchKernelExC(&cfg, e->kernels.adjoint, args));
  return PGA_OK;
}

extern "C" PgaStatus pga_adjoint(PgaEngine* e, const float* dGradTerminals, float* dGradParams, uint32_t numBlocks,
                                 float* dGradAxiomSizes, void* stream) {
  return pga_adjoint_strided(e, dGradTerminals, 12u, dGradParams, numBlocks, dGradAxiomSizes, stream);
}
#endif  // PGA_ADJOINT_DEVICE_ONLY
