// Adjoint of the derivation (no reference counterpart).
//
// With the discrete derivation frozen -- every IfSizeLess branch, Repeat count,
// discard and the rule of every shape as recorded by the forward pass -- a
// terminal's transform is a smooth function of the continuous inputs: the
// per-axiom parameter blocks (PGA_PT_BLOCK parameters) and the axiom sizes.
// Rotations are signed permutations that no continuous input changes, so the
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

struct Grad {
  float t[3], s[3];
};

__device__ __forceinline__ void grad_zero(Grad& g) {
#pragma unroll
  for (int k = 0; k < 3; k++) g.t[k] = g.s[k] = 0.0f;
}

struct AdjArgs {
  const float* gradTerminals;  // 12 per terminal
  float* gradParams;           // numBlocks * blockStride
  uint32_t numBlocks;
  float* gradSizes;            // 3 per axiom
  float* nodeGrad;             // 6 per item: d/dt, d/ds
  unsigned long long numTerminals;
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
    if (j.gradParams != nullptr && slot < a.blockStride && b < j.numBlocks)
      atomicAdd(&j.gradParams[(size_t)b * a.blockStride + slot], g);
  } else if (p.type == PGA_PT_SHAPE_ATTR && gx != nullptr) {
    const uint32_t i = f2u(p.v0);
    if (i >= 12 && i < 15) gx->s[i - 12] += g;
    if (i < 12 && (i & 3u) == 3u) gx->t[i >> 2] += g;
  } else if (p.type == PGA_PT_EXP && gx != nullptr) {
    exp_grad(a.tab.expPool + p.aux, x, __ldg(&a.axioms[x.axiom].custom), g, *gx);
  }
}

// d(offset along the split axis) seen through the translation: R[:,a] has one
// nonzero entry, +-1 in row perm_a.
__device__ __forceinline__ float axis_dot(const Shape& x, uint32_t ax, const float gt[3]) {
  const float v = pick3(gt, frame_row(x.frame, ax));
  return frame_neg(x.frame, ax) ? -v : v;
}

// VJP of child c of the item held in E (state before producing children,
// i.e. right after expander_init).  gc is the gradient of the child's state;
// the parent's gradient is accumulated into gp.
__device__ void child_vjp(const DeriveArgs& a, const AdjArgs& j, const Expander& E0, uint32_t c, const Grad& gc,
                          Grad& gp) {
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
      const float go = axis_dot(x, ax, gc.t);
      for (uint32_t k = 0; k < 3; k++)
        if (k != ax) gp.s[k] += gc.s[k];
      // Reverse pass over the recurrence that produced child c:
      //   offset_0 = -S/2;  N_i = size(f_i, scale);  o_i = offset_i + N_i/2;
      //   offset_{i+1} = offset_i + N_i;  child c: size N_c, translation t + R_a o_c.
      // Factor f_i is read on the base shape (static form, i = 0, or a rule
      // whose factors do not read the shape) or, for a dynamic Subdivide, on the
      // symbol as child i - 1 left it in place: size N_{i-1} along a and
      // translation t + R_a o_{i-1}; its gradient then flows to N_{i-1},
      // o_{i-1} and the base's other sizes and translation.  The scale uses
      // the factors read from the base shape.
      constexpr uint32_t kMaxN = PGA_MAX_NUM_PARAMETERS;
      float fv[kMaxN], Nv[kMaxN], ov[kMaxN], gN[kMaxN], goI[kMaxN];
      const uint32_t last = min(c, n - 1u);
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
        gN[i] = 0.0f;
        goI[i] = 0.0f;
      }
      if (last >= kMaxN) return;
      gN[last] += pick3(gc.s, ax);
      goI[last] += go;
      const bool readsUpdated = dyn && !(r.flags & kRulePure);
      float gS = 0.0f, gscale = 0.0f, gOffNext = 0.0f;
      for (int i = (int)last; i >= 0; i--) {
        // o_i = offset_i + N_i/2 and offset_{i+1} = offset_i + N_i
        const float gOff = gOffNext + goI[i];
        gN[i] += gOffNext + 0.5f * goI[i];
        gOffNext = gOff;
        const float f = fv[i];
        if (!dyn && f == 0.0f) continue;  // a skipped static slot
        float gf = 0.0f;
        if (f > 0.0f) {
          gf = gN[i];
        } else if (f < 0.0f) {
          gf = gN[i] * (-E0.scale);
          gscale += gN[i] * (-f);
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
          gN[i - 1] += pick3(gst.s, ax);
          for (uint32_t k = 0; k < 3; k++)
            if (k != ax) gp.s[k] += gst.s[k];
#pragma unroll
          for (int q = 0; q < 3; q++) gp.t[q] += gst.t[q];
          goI[i - 1] += axis_dot(x, ax, gst.t);
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
      if (ext < 0.0f) {
        gS += gE * fabsf(ext);
        param_grad(a, j, r, 1, x, gE * (-S), &gp);
      } else {
        param_grad(a, j, r, 1, x, gE, &gp);
      }
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

// Recomputes the shape created as child `ordinal` of `link` (an item or an
// axiom) and replays its 1 -> 1 chain until `stopAt` (a terminal: the Generate
// rule; an item: its branching rule).  The smooth steps (Extrude, Translate,
// Scale, SwapSize) are recorded so that the reverse pass can undo them; a chain with
// more than kChainSteps of them has no adjoint (PGA_ERR_NO_TAPE).
constexpr int kChainSteps = 8;
struct Chain {
  uint32_t n;                   // smooth steps
  int32_t entry[kChainSteps];   // rule of each step
  Shape before[kChainSteps];    // state entering each step
};

__device__ bool replay(const DeriveArgs& a, uint32_t link, uint32_t ordinal, bool toTerminal, Expander& E,
                       bool& fromAxiom, uint32_t& c, Shape& y0, Chain& ch, Shape& yEnd) {
  fromAxiom = (link & kAxiomLink) != 0;
  if (fromAxiom) {
    axiom_shape(a, link & ~kAxiomLink, y0);
    c = 0;
  } else {
    uint4 ext;
    load_node(a, link, E.base, ext);
    const int32_t e = E.base.entry;
    if (e < 0 || (uint32_t)e >= a.tab.numEntries) return false;
    E.r = rule_at(a, (uint32_t)e);
    E.base.kind = E.r.shape;
    const uint32_t all = expander_init(a, E);
    c = (E.r.op == PGA_OP_REPEAT) ? ordinal - 1u : ordinal;
    if (c >= all) return false;
    Expander W = E;
    expander_skip(a, W, c);
    uint32_t ord;
    if (!expander_child(a, W, c, y0, ord)) return false;
  }
  ch.n = 0;
  Shape x = y0;
  for (int step = 0; step < kMaxChain; step++) {
    if (x.entry < 0 || (uint32_t)x.entry >= a.tab.numEntries) return false;
    const DevRule r = rule_at(a, (uint32_t)x.entry);
    if (r.op == PGA_OP_IF_SIZE_LESS) {
      uint32_t axis;
      if (!axis_param(a, r, x, axis)) return false;
      const float size = param(a, r, 1, x);
      const uint32_t branch = (pick3(x.s, axis) < size) ? 0u : 1u;
      x.path = child_path(x.path, branch, succ_at(a, r.succBase + branch));
      x.entry = succ_at(a, r.succBase + branch);
      continue;
    }
    if (r.op == PGA_OP_RANDOM_RULE || r.op == PGA_OP_RANDOM_RULE_STATIC) {
      const int pick = random_pick(a, r, x);
      if (pick < 0) return false;
      const int32_t nxt = succ_at(a, r.succBase + (uint32_t)pick);
      x.path = child_path(x.path, (uint32_t)pick, nxt);
      x.entry = nxt;
      continue;
    }
    if (r.op == PGA_OP_IF) {
      const uint32_t branch = (param(a, r, 0, x) != 0.0f) ? 0u : 1u;
      x.path = child_path(x.path, branch, succ_at(a, r.succBase + branch));
      x.entry = succ_at(a, r.succBase + branch);
      continue;
    }
    if (r.op == PGA_OP_TRANSLATE || r.op == PGA_OP_SCALE || r.op == PGA_OP_SWAP_SIZE) {
      if (ch.n >= kChainSteps) return false;
      ch.entry[ch.n] = x.entry;
      ch.before[ch.n] = x;
      ch.n++;
      if (r.op == PGA_OP_TRANSLATE)
        apply_translate(a, r, x);
      else if (r.op == PGA_OP_SCALE)
        apply_scale(a, r, x);
      else if (!swap_size(a, r, x))
        return false;
      x.entry = succ_at(a, r.succBase);
      continue;
    }
    if (r.op == PGA_OP_EXTRUDE) {
      if (ch.n >= kChainSteps) return false;
      ch.entry[ch.n] = x.entry;
      ch.before[ch.n] = x;
      ch.n++;
      const float extent = param(a, r, 1, x);
      const uint32_t f = x.frame;
      x.frame = frame_set(frame_set(f, 1, f, 2, 0), 2, f, 1, 1);
      x.s[2] = x.s[1];
      x.s[1] = extent;
      x.seed = seed_of(a, x.seed, 0u);
      x.kind = PGA_SHAPE_BOX;
      const int32_t nxt = succ_at(a, r.succBase);
      x.path = child_path(x.path, 0u, nxt);
      x.entry = nxt;
      continue;
    }
    const bool isTerm = r.op == PGA_OP_GENERATE;
    yEnd = x;
    return isTerm == toTerminal;
  }
  return false;
}

// Pushes the gradient g of a record, whose creation has been replayed into
// (E, fromAxiom, c, ch), back to its parent.
__device__ void push_back_replayed(const DeriveArgs& a, const AdjArgs& j, uint32_t link, const Expander& E,
                                   bool fromAxiom, uint32_t c, const Chain& ch, Grad g) {
  // Undo the smooth steps, last first.
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
  if (fromAxiom) {
    const uint32_t ax = link & ~kAxiomLink;
    if (j.gradSizes != nullptr)
      for (int q = 0; q < 3; q++)
        if (g.s[q] != 0.0f) atomicAdd(&j.gradSizes[(size_t)ax * 3 + q], g.s[q]);
    return;
  }
  Grad gp;
  grad_zero(gp);
  child_vjp(a, j, E, c, g, gp);
  float* dst = j.nodeGrad + (size_t)link * 6;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    if (gp.t[q] != 0.0f) atomicAdd(dst + q, gp.t[q]);
    if (gp.s[q] != 0.0f) atomicAdd(dst + 3 + q, gp.s[q]);
  }
}

// Pushes the gradient g of the recorded record back to its parent.
__device__ void push_back(const DeriveArgs& a, const AdjArgs& j, uint32_t link, uint32_t ordinal, bool toTerminal,
                          Grad g) {
  Expander E;
  bool fromAxiom;
  uint32_t c;
  Shape y0, yEnd;
  Chain ch;
  if (!replay(a, link, ordinal, toTerminal, E, fromAxiom, c, y0, ch, yEnd)) {
    raise_error(a.st, PGA_ERR_NO_TAPE, (int)link);
    return;
  }
  push_back_replayed(a, j, link, E, fromAxiom, c, ch, g);
}

// Reverse step of terminal t: dL/dM (12 floats) to the gradient of the
// Generate rule's shape, then back to its parent.
__device__ __forceinline__ void adj_terminal(const DeriveArgs& a, const AdjArgs& j, unsigned long long t) {
  const float* gm = j.gradTerminals + t * 12;
  const uint2 link = a.termLinks[t];
  Grad g;
  float G[12];
#pragma unroll
  for (int q = 0; q < 12; q++) G[q] = __ldg(gm + q);
  // Generate: M[:, k] = R[:, k] s_k and M[:, 3] = t, with R from the replayed state.
  Expander E;
  bool fromAxiom;
  uint32_t c;
  Shape y0, yEnd;
  Chain ch;
  if (!replay(a, link.x, link.y, true, E, fromAxiom, c, y0, ch, yEnd)) {
    raise_error(a.st, PGA_ERR_NO_TAPE, (int)t);
    return;
  }
#pragma unroll
  for (int q = 0; q < 3; q++) {
    g.t[q] = G[q * 4 + 3];
    const uint32_t row = frame_row(yEnd.frame, q);
    const float v = G[row * 4 + q];
    g.s[q] = frame_neg(yEnd.frame, q) ? -v : v;
  }
  push_back_replayed(a, j, link.x, E, fromAxiom, c, ch, g);
}

// Reverse step of work item i: its accumulated gradient back to its parent.
__device__ __forceinline__ void adj_item(const DeriveArgs& a, const AdjArgs& j, unsigned long long i) {
  const uint4 ext = __ldcg(reinterpret_cast<const uint4*>(a.nodes + i) + 3);
  if (ext.x == kEmptyItem) return;
  Grad g;
  const float* src = j.nodeGrad + i * 6;
  bool any = false;
#pragma unroll
  for (int q = 0; q < 3; q++) {
    g.t[q] = __ldcg(src + q);
    g.s[q] = __ldcg(src + 3 + q);
    any |= (g.t[q] != 0.0f) || (g.s[q] != 0.0f);
  }
  if (any) push_back(a, j, ext.z, ext.w, false, g);
}

// The whole reverse sweep in one cooperative launch: zero the accumulators and
// outputs, visit every terminal, then the levels from the deepest up, with a
// bounded grid barrier after each phase.  The level bounds, the item and the
// terminal counts are the forward launch's final state, read on the device,
// so no host round trip is needed.  A failed or overflowed forward pass leaves
// the gradients zero (the engine report keeps the forward's status; a tape
// too short for the terminals raises PGA_ERR_NO_TAPE).
__global__ void __launch_bounds__(kThreads) k_adjoint(DeriveArgs a, AdjArgs j, unsigned long long numParamFloats,
                                                      uint32_t numAxioms) {
  Smem& sm = *reinterpret_cast<Smem*>(smem_raw);
  setup_block(a, sm);
  volatile DevState* vs = a.st;
  // Fixed by the forward launch; nothing below changes them before the first barrier.
  const unsigned long long nodes = min((unsigned long long)vs->nodeNext, a.nodeCap);
  const unsigned long long nTerm = vs->termCount;
  const uint32_t levels = vs->levels;
  const bool ok = vs->status == 0 && nTerm <= a.cap && nTerm <= a.termLinkCap;
  const unsigned long long tid = (unsigned long long)blockIdx.x * kThreads + threadIdx.x;
  const unsigned long long stride = (unsigned long long)gridDim.x * kThreads;
  for (unsigned long long k = tid; k < nodes * 6; k += stride) j.nodeGrad[k] = 0.0f;
  if (j.gradParams)
    for (unsigned long long k = tid; k < numParamFloats; k += stride) j.gradParams[k] = 0.0f;
  if (j.gradSizes)
    for (unsigned long long k = tid; k < (unsigned long long)numAxioms * 3; k += stride) j.gradSizes[k] = 0.0f;
  if (!grid_barrier(a, [] {})) return;
  if (!ok) {
    if (tid == 0 && vs->status == 0) raise_error(a.st, PGA_ERR_NO_TAPE, -1);
    return;
  }
  for (unsigned long long t = tid; t < nTerm; t += stride) adj_terminal(a, j, t);
  if (!grid_barrier(a, [] {})) return;
  for (int L = (int)levels; L >= 0; L--) {
    const unsigned long long lo = a.levelStart[L], hi = min(a.levelStart[L + 1], nodes);
    for (unsigned long long i = lo + tid; i < hi; i += stride) adj_item(a, j, i);
    if (!grid_barrier(a, [] {})) return;
  }
}

}  // namespace pga

extern "C" PgaStatus pga_adjoint(PgaEngine* e, const float* dGradTerminals, float* dGradParams, uint32_t numBlocks,
                                 float* dGradAxiomSizes, void* stream) {
  using namespace pga;
  if (!e || !dGradTerminals) {
    set_error("pga_adjoint: null engine or gradient");
    return PGA_ERR_INVALID_ARGUMENT;
  }
  if (!e->cfg.recordTape || !e->lastWasBatched || !e->dTermLinks || !e->lastOut) {
    set_error("pga_adjoint: the last derivation was not a pga_derive on an engine created with recordTape = 1");
    return PGA_ERR_NO_TAPE;
  }
  if (e->adjointBlocks == 0) {
    // One cooperative launch: as many blocks as can be resident with the
    // engine's dynamic shared memory.
    PGA_CUDA_TRY(cudaFuncSetAttribute(k_adjoint, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e->smemBytes));
    int perSM = 0;
    PGA_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, k_adjoint, kThreads, e->smemBytes));
    if (perSM < 1) {
      set_error("pga_adjoint: the adjoint kernel does not fit on an SM");
      return PGA_ERR_CUDA;
    }
    e->adjointBlocks = perSM * e->numSMs;
  }
  DeriveArgs a = make_args(e, e->lastAxioms, e->lastNumAxioms, e->lastBlocks, e->lastOut, e->lastCap, nullptr);
  AdjArgs j;
  j.gradTerminals = dGradTerminals;
  j.gradParams = dGradParams;
  j.numBlocks = numBlocks;
  j.gradSizes = dGradAxiomSizes;
  j.nodeGrad = e->dNodeGrad;
  j.numTerminals = 0;  // read on the device
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
  PGA_CUDA_TRY(cudaLaunchKernelExC(&cfg, (const void*)k_adjoint, args));
  return PGA_OK;
}
