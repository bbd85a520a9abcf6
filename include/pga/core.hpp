/*
 * pga/core.hpp -- C++ grammar front end of the GB300 derivation engine.
 *
 * The reference's grammar vocabulary, with the same names and template
 * parameters, so that a procedure list written for the reference compiles
 * unchanged against this header:
 *   - PGA::Proc<ShapeT, OperatorT, NumThreadsT>           (include/pga/core/Proc.cuh:19-27)
 *   - PGA::Shapes::Box, Quad                              (include/pga/core/Shapes.cuh)
 *   - PGA::Operators::Subdivide, Repeat, ComponentSplit, Extrude, IfSizeLess,
 *     Generate, Discard, Translate, Rotate, Scale, RandomRule, Replicate, If,
 *     SwapSize, Collider, IfCollides
 *                                                          (Subdivide.cuh:22,170; Repeat.cuh:35-64;
 *                                                          ComponentSplit.cuh:234-270; Extrude.cuh:24;
 *                                                          If.cuh:60; Generate.cuh:23-49; Discard.cuh:15;
 *                                                          Translate.cuh:24; Rotate.cuh:21; Scale.cuh:23;
 *                                                          RandomRule.cuh:20,121; Replicate.cuh:19,92;
 *                                                          If.cuh:22; SwapSize.cuh:20)
 *   - PGA::Operators::DCall, PSCall, FSCall                (Call.cuh:23-346)
 *   - PGA::Parameters::DynParam, DynParams, Scalar, AxisParam, RepeatModeParam,
 *     ShapeAttr, ShapePos, ShapeRotation, ShapeNormal, ShapeSize, ShapeSeed,
 *     ShapeCustomAttribute, Rand, Exp and the expression operators
 *                                                          (Parameters.cuh:28-817)
 *   - T::List, T::Pair                                     (include/pga/core/TStdLib.h)
 *   - PGA::DispatchTable with Parameter / Successor / Entry (DispatchTable.h:16-98)
 *
 * These templates carry no device code.  PGA::lower<ProcedureList>(table)
 * turns a procedure list plus a dispatch table into the engine's rule table
 * (PgaProc list + PgaEntry array, include/pga_gb300.h) on the host:
 *   - DynParam<i> reads parameter i of the dispatch entry being lowered, a
 *     static parameter becomes the parameter its reference toParameter() gives
 *     (Scalar -> PT_SCALAR, Rand -> PT_RAND, ShapeAttr -> PT_SHAPE_ATTR,
 *     Exp -> PT_EXP in the reference's postfix encoding);
 *   - DCall<k> / PSCall<op, k> follow successor k of that entry, FSCall<op,
 *     phase, -1, e> goes to entry e;
 *   - an operator used directly as a successor (a static chain such as
 *     Subdivide<..., T::Pair<Scalar<-1>, Generate<...>>>) becomes an extra
 *     rule-table entry appended after the dispatch table's own entries.  Its
 *     DynParam / DCall arguments keep reading the entry that started the chain,
 *     as in the reference, where the default SymbolDecorator leaves the child's
 *     entry index unchanged (SymbolDecorator.cuh:11-20).
 * Entry i of the dispatch table stays entry i of the rule table, so axioms
 * keep their root entries.
 *
 * Generate<..., 1, ...> is an instanced terminal, Generate<..., 0, ...> a
 * triangle-mesh terminal (PGA_OP_GENERATE_MESH, expanded by
 * pga_generate_meshes).  Not lowered (an exception names them): other
 * generation functions, the Vec2/Vec4 parameter types, FSCall without an entry
 * index, and the operators outside this engine (the SetAs prism and polygon
 * operators).  Generate's Attr1..Attr5 arguments are accepted and
 * unused: the instanced generation function writes the shape's custom
 * attribute (GenerationFunctions.cuh:158-188).
 */
#ifndef PGA_GB300_CORE_HPP
#define PGA_GB300_CORE_HPP

#include <pga_gb300.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <initializer_list>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace T {
template <typename... ItemsT>
struct List {};
template <typename FirstT, typename SecondT>
struct Pair {};
}  // namespace T

namespace PGA {

enum Axis { X = 0, Y, Z };
enum RepeatMode { ANCHOR_TO_START = 0, ANCHOR_TO_END, ADJUST_TO_FILL };
enum ParameterType { PT_SCALAR = 0, PT_RAND, PT_SHAPE_ATTR, PT_EXP, PT_VEC2, PT_VEC4 };
enum OperationType { OPT_ADD = 0, OPT_SUB, OPT_DIV, OPT_MULTI, OPT_EQ, OPT_NEQ, OPT_LT, OPT_GT, OPT_LEQ, OPT_GEQ, OPT_AND, OPT_OR };
enum OperandType { ORT_SCALAR = 0, ORT_RAND, ORT_SHAPE_ATTR, ORT_OP };

class LoweringError : public std::runtime_error {
 public:
  explicit LoweringError(const std::string& what) : std::runtime_error("PGA::lower: " + what) {}
};

// ------------------------------------------------------------ dispatch table

/* Grammar data, built with the same brace syntax as the reference's
 * PGA::DispatchTable: { operatorCode, { {type, {values}}... }, { {entry, phase}... } }. */
struct DispatchTable {
  struct Parameter {
    ParameterType type;
    std::vector<double> values;
    Parameter() : type(PT_SCALAR) {}
    Parameter(ParameterType t, const std::vector<double>& v) : type(t), values(v) {}
    Parameter(ParameterType t, std::initializer_list<double> v) : type(t), values(v) {}
    PgaParameter toParameter() const {
      if (values.size() > PGA_MAX_NUM_PARAMETER_VALUES) throw LoweringError("too many parameter values");
      PgaParameter p;
      std::memset(&p, 0, sizeof p);
      p.type = (int32_t)type;
      for (size_t i = 0; i < values.size(); i++) p.value[i] = (float)values[i];
      return p;
    }
  };
  struct Successor {
    int entryIndex, phaseIndex;
    Successor() : entryIndex(-1), phaseIndex(-1) {}
    Successor(int entry, int phase) : entryIndex(entry), phaseIndex(phase) {}
  };
  struct Entry {
    size_t operatorCode;
    std::vector<Parameter> parameters;
    std::vector<Successor> successors;
    std::vector<int> edgeIndices;  // instrumentation only; not used by the engine
    int subGraphIndex;
    Entry() : operatorCode(0), subGraphIndex(-1) {}
    Entry(size_t code, std::initializer_list<Parameter> params, std::initializer_list<Successor> succs,
          std::initializer_list<int> edges = {}, int subGraph = -1)
        : operatorCode(code), parameters(params), successors(succs), edgeIndices(edges), subGraphIndex(subGraph) {}
    PgaEntry toEntry() const {
      if (parameters.size() > PGA_MAX_NUM_PARAMETERS) throw LoweringError("too many parameters");
      if (successors.size() > PGA_MAX_NUM_SUCCESSORS) throw LoweringError("too many successors");
      PgaEntry e;
      std::memset(&e, 0, sizeof e);
      e.operatorCode = (int32_t)operatorCode;
      e.numParameters = (uint32_t)parameters.size();
      for (size_t i = 0; i < parameters.size(); i++) e.parameters[i] = parameters[i].toParameter();
      e.numSuccessors = (uint32_t)successors.size();
      for (size_t i = 0; i < PGA_MAX_NUM_SUCCESSORS; i++) {
        e.successors[i].entryIndex = i < successors.size() ? successors[i].entryIndex : -1;
        e.successors[i].phaseIndex = i < successors.size() ? successors[i].phaseIndex : -1;
      }
      return e;
    }
  };

  std::vector<Entry> entries;
  DispatchTable() = default;
  DispatchTable(std::initializer_list<Entry> e) : entries(e) {}

  std::vector<PgaEntry> toEntries() const {
    std::vector<PgaEntry> out;
    out.reserve(entries.size());
    for (const Entry& e : entries) out.push_back(e.toEntry());
    return out;
  }
};

// -------------------------------------------------------------------- shapes

namespace Shapes {
struct Box {
  static constexpr uint32_t kind = PGA_SHAPE_BOX;
};
struct Quad {
  static constexpr uint32_t kind = PGA_SHAPE_QUAD;
};
}  // namespace Shapes

// ---------------------------------------------------------------- parameters

namespace detail {
constexpr unsigned long long pow10(unsigned n) { return n == 0 ? 1ull : 10ull * pow10(n - 1); }

inline PgaParameter make_parameter(uint32_t type, float v0 = 0.0f, float v1 = 0.0f) {
  PgaParameter p;
  std::memset(&p, 0, sizeof p);
  p.type = (int32_t)type;
  p.value[0] = v0;
  p.value[1] = v1;
  return p;
}

// An operand word of an expression program: operand type in the top two bits,
// the value's bits shifted right by two below (PackUtils::packOperand, PackUtils.h:18-23).
inline float pack_operand(OperandType t, float x) {
  uint32_t r;
  std::memcpy(&r, &x, 4);
  const uint32_t q = (r >> 2) | ((uint32_t)t << 30);
  float f;
  std::memcpy(&f, &q, 4);
  return f;
}

// Two values in [0, 1] quantised to 12 bits each in one float (PackUtils::packFloat2, PackUtils.h:25-28).
inline float pack_float2(float x, float y) {
  return std::floor(x * 4095.0f) * 4096.0f + std::floor(y * 4095.0f);
}
}  // namespace detail

namespace Parameters {

/* Parameter i of the dispatch entry being executed (Parameters.cuh:744-815). */
template <unsigned int ParamIdxT>
struct DynParam {
  static const unsigned int Length = 1;
};

/* Marker of Subdivide<DynParams>: axis and factors come from the entry (Parameters.cuh:817). */
class DynParams {};

template <int ValueT, unsigned int NegativeOrderOfMagnitudeT = 0>
struct Scalar {
  static const unsigned int Length = 1;
  static float getValue() { return (float)ValueT / (float)detail::pow10(NegativeOrderOfMagnitudeT); }
  static PgaParameter toParameter() { return detail::make_parameter(PGA_PT_SCALAR, getValue()); }
  static void encode(float* b, unsigned int p) { b[p] = detail::pack_operand(ORT_SCALAR, getValue()); }
};

template <Axis AxisT>
struct AxisParam : Scalar<AxisT, 0> {};

template <RepeatMode RepeatModeT>
struct RepeatModeParam : Scalar<RepeatModeT, 0> {};

/* Shape attribute i: 0..11 model rows, 12..14 size, 15 seed, 16 custom attribute (Shape.cuh:120-171). */
template <unsigned int IndexT>
struct ShapeAttr {
  static const unsigned int Length = 1;
  static PgaParameter toParameter() { return detail::make_parameter(PGA_PT_SHAPE_ATTR, (float)IndexT); }
  static void encode(float* b, unsigned int p) { b[p] = detail::pack_operand(ORT_SHAPE_ATTR, (float)IndexT); }
};

template <Axis AxisT>
struct ShapePos : ShapeAttr<(AxisT + 1) * 4 - 1> {};
template <Axis AxisT, Axis ComponentT>
struct ShapeRotation : ShapeAttr<(ComponentT * 4) + AxisT> {};
template <Axis ComponentT>
struct ShapeNormal : ShapeRotation<Z, ComponentT> {};
template <Axis AxisT>
struct ShapeSize : ShapeAttr<AxisT + 12> {};
struct ShapeSeed : ShapeAttr<15> {};
struct ShapeCustomAttribute : ShapeAttr<16> {};

template <int MinT, int MaxT, unsigned int MinNegativeOrderOfMagnitudeT = 0, unsigned int MaxNegativeOrderOfMagnitudeT = 0>
struct Rand {
  static const unsigned int Length = 1;
  static float getMin() { return (float)MinT / (float)detail::pow10(MinNegativeOrderOfMagnitudeT); }
  static float getMax() { return (float)MaxT / (float)detail::pow10(MaxNegativeOrderOfMagnitudeT); }
  static PgaParameter toParameter() { return detail::make_parameter(PGA_PT_RAND, getMin(), getMax()); }
  static void encode(float* b, unsigned int p) {
    b[p] = detail::pack_operand(ORT_RAND, detail::pack_float2(getMin(), getMax()));
  }
};

/* Binary expression node: both operands in postfix order, then the operation. */
template <typename OperandAT, typename OperandBT, OperationType OpTypeT>
struct ExpOperator {
  static const unsigned int Length = OperandAT::Length + OperandBT::Length + 1;
  static void encode(float* b, unsigned int p) {
    OperandAT::encode(b, p);
    OperandBT::encode(b, p + OperandAT::Length);
    b[p + OperandAT::Length + OperandBT::Length] = detail::pack_operand(ORT_OP, (float)OpTypeT);
  }
};

template <typename A, typename B> struct Add : ExpOperator<A, B, OPT_ADD> {};
template <typename A, typename B> struct Sub : ExpOperator<A, B, OPT_SUB> {};
template <typename A, typename B> struct Multi : ExpOperator<A, B, OPT_MULTI> {};
template <typename A, typename B> struct Div : ExpOperator<A, B, OPT_DIV> {};
template <typename A, typename B> struct Eq : ExpOperator<A, B, OPT_EQ> {};
template <typename A, typename B> struct Neq : ExpOperator<A, B, OPT_NEQ> {};
template <typename A, typename B> struct Lt : ExpOperator<A, B, OPT_LT> {};
template <typename A, typename B> struct Gt : ExpOperator<A, B, OPT_GT> {};
template <typename A, typename B> struct Leq : ExpOperator<A, B, OPT_LEQ> {};
template <typename A, typename B> struct Geq : ExpOperator<A, B, OPT_GEQ> {};
template <typename A, typename B> struct And : ExpOperator<A, B, OPT_AND> {};
template <typename A, typename B> struct Or : ExpOperator<A, B, OPT_OR> {};

/* Expression parameter: value[0] = program length, value[1..] = the postfix
 * program (Parameters.cuh:459-483). */
template <typename OperandAT, typename OperandBT, template <class, class> class OpT>
struct Exp {
  static const unsigned int Length = OperandAT::Length + OperandBT::Length + 1;
  static PgaParameter toParameter() {
    static_assert(Length + 1 <= PGA_MAX_NUM_PARAMETER_VALUES, "expression longer than a parameter holds");
    PgaParameter p = detail::make_parameter(PGA_PT_EXP, (float)Length);
    OpT<OperandAT, OperandBT>::encode(p.value + 1, 0);
    return p;
  }
  static void encode(float* b, unsigned int p) { OpT<OperandAT, OperandBT>::encode(b, p); }
};

}  // namespace Parameters

// ----------------------------------------------------------------- operators

namespace Operators {

template <unsigned int SuccessorOffsetT, int EdgeIndexT = -1>
class DCall {};
template <unsigned int OperationCodeT, unsigned int SuccessorOffsetT, int EdgeIndexT = -1>
class PSCall {};
template <unsigned int OperationCodeT, int PhaseIndexT, int EdgeIndexT = -1, int EntryIndexT = -1>
class FSCall {};

template <typename AxisT, typename... Params1T>
class Subdivide {};
template <bool ParallelT, typename AxisT, typename ExtentT, typename RepeatModeT, typename NextOperatorT>
class Repeat {};
template <bool ParallelT, typename TopOperatorT, typename BottomOperatorT, typename SidesOperatorT>
class ComponentSplit {};
template <typename AxisT, typename ExtentT, typename NextOperatorT>
class Extrude {};
template <typename AxisT, typename SizeT, typename NextOperatorIfTrueT, typename NextOperatorIfFalseT>
class IfSizeLess {};
template <bool ParallelT, unsigned int GenFuncIdxT = 0, typename TerminalIdxT = Parameters::Scalar<0>,
          typename Attr1T = Parameters::Scalar<0>, typename Attr2T = Parameters::Scalar<0>,
          typename Attr3T = Parameters::Scalar<0>, typename Attr4T = Parameters::Scalar<0>,
          typename Attr5T = Parameters::Scalar<0>>
class Generate {};
class Discard {};
template <typename XT, typename YT, typename ZT, typename NextOperatorT>
class Translate {};
template <typename XT, typename YT, typename ZT, typename NextOperatorT>
class Rotate {};
template <typename XT, typename YT, typename ZT, typename NextOperatorT>
class Scale {};
template <typename ChanceT, typename... Params1T>
class RandomRule {};
template <typename... Params1T>
class Replicate {};
template <typename ExpressionT, typename NextOperatorIfTrueT, typename NextOperatorIfFalseT>
class If {};
template <typename XT, typename YT, typename ZT, typename NextOperatorT>
class SwapSize {};
template <typename ColliderTagT, typename NextOperatorT>
class Collider {};
template <typename ColliderTagT, typename NextOperatorIfTrueT, typename NextOperatorIfFalseT>
class IfCollides {};

}  // namespace Operators

template <typename ShapeT, typename OperatorT, unsigned int NumThreadsT = 1>
class Proc {};

// ------------------------------------------------------------------ lowering

/* The engine's rule table produced by lower(): procedures plus entries; view()
 * gives the PgaRuleTable for pga_engine_create (valid while this object lives). */
struct LoweredTable {
  std::vector<PgaProc> procs;
  std::vector<PgaEntry> entries;
  uint32_t numUserEntries = 0;  // entries [0, numUserEntries) are the dispatch table's own
  PgaRuleTable view() const {
    PgaRuleTable t;
    t.procs = procs.data();
    t.numProcs = (uint32_t)procs.size();
    t.entries = entries.data();
    t.numEntries = (uint32_t)entries.size();
    return t;
  }
};

namespace detail {

class Builder {
 public:
  LoweredTable out;

  uint32_t proc(uint32_t op, uint32_t shape, uint32_t numChildren) {
    const auto key = std::make_tuple(op, shape, numChildren);
    auto it = index_.find(key);
    if (it != index_.end()) return it->second;
    const uint32_t i = (uint32_t)out.procs.size();
    out.procs.push_back(PgaProc{op, shape, numChildren, 1u});
    index_.emplace(key, i);
    return i;
  }
  uint32_t new_entry() {
    if (out.entries.size() >= (size_t)INT32_MAX) throw LoweringError("rule table too large");
    PgaEntry e;
    std::memset(&e, 0, sizeof e);
    for (auto& s : e.successors) s.entryIndex = s.phaseIndex = -1;
    out.entries.push_back(e);
    return (uint32_t)out.entries.size() - 1;
  }

 private:
  std::map<std::tuple<uint32_t, uint32_t, uint32_t>, uint32_t> index_;
};

// Parameter lowering: a static parameter's own toParameter(), DynParam<i> the entry's parameter i.
template <typename ParamT>
struct LowerParam {
  static PgaParameter run(const PgaEntry&) { return ParamT::toParameter(); }
};
template <unsigned int I>
struct LowerParam<Parameters::DynParam<I>> {
  static PgaParameter run(const PgaEntry& src) {
    if (I >= src.numParameters)
      throw LoweringError("DynParam<" + std::to_string(I) + "> beyond the entry's " +
                          std::to_string(src.numParameters) + " parameters");
    return src.parameters[I];
  }
};

template <typename OperatorT, typename ShapeT>
struct LowerOp {
  static void run(Builder&, const PgaEntry&, uint32_t) {
    throw LoweringError("operator not supported by the GB300 engine");
  }
};

// Successor lowering: a call follows the entry's successor table, an operator
// becomes a new entry (same source entry) for the child's shape.
template <typename SuccT, typename ShapeT>
struct LowerSucc {
  static PgaSuccessor run(Builder& b, const PgaEntry& src) {
    const uint32_t i = b.new_entry();
    LowerOp<SuccT, ShapeT>::run(b, src, i);
    return PgaSuccessor{(int32_t)i, 0};
  }
};
inline PgaSuccessor successor_of(const PgaEntry& src, unsigned int k) {
  if (k >= src.numSuccessors)
    throw LoweringError("successor " + std::to_string(k) + " beyond the entry's " + std::to_string(src.numSuccessors) +
                        " successors");
  return src.successors[k];
}
template <unsigned int K, int E, typename ShapeT>
struct LowerSucc<Operators::DCall<K, E>, ShapeT> {
  static PgaSuccessor run(Builder&, const PgaEntry& src) { return successor_of(src, K); }
};
template <unsigned int Op, unsigned int K, int E, typename ShapeT>
struct LowerSucc<Operators::PSCall<Op, K, E>, ShapeT> {
  static PgaSuccessor run(Builder&, const PgaEntry& src) { return successor_of(src, K); }
};
template <unsigned int Op, int Phase, int E, int Entry, typename ShapeT>
struct LowerSucc<Operators::FSCall<Op, Phase, E, Entry>, ShapeT> {
  static PgaSuccessor run(Builder&, const PgaEntry&) {
    if (Entry < 0) throw LoweringError("FSCall without an entry index");
    return PgaSuccessor{Entry, Phase};
  }
};

// Writes entry i once its parameters and successors are known (appending
// nested entries may move the vector, so the entry is filled last).
inline void set_entry(Builder& b, uint32_t i, uint32_t proc, const std::vector<PgaParameter>& params,
                      const std::vector<PgaSuccessor>& succs) {
  if (params.size() > PGA_MAX_NUM_PARAMETERS || succs.size() > PGA_MAX_NUM_SUCCESSORS)
    throw LoweringError("entry exceeds the parameter or successor limit");
  PgaEntry& e = b.out.entries[i];
  e.operatorCode = (int32_t)proc;
  e.numParameters = (uint32_t)params.size();
  for (size_t k = 0; k < params.size(); k++) e.parameters[k] = params[k];
  e.numSuccessors = (uint32_t)succs.size();
  for (size_t k = 0; k < succs.size(); k++) e.successors[k] = succs[k];
}

template <typename... PairsT>
struct StaticPairs;
template <>
struct StaticPairs<> {
  template <typename ShapeT>
  static void run(Builder&, const PgaEntry&, std::vector<PgaParameter>&, std::vector<PgaSuccessor>&) {}
};
template <typename FactorT, typename SuccT, typename... RestT>
struct StaticPairs<T::Pair<FactorT, SuccT>, RestT...> {
  template <typename ShapeT>
  static void run(Builder& b, const PgaEntry& src, std::vector<PgaParameter>& params, std::vector<PgaSuccessor>& succs) {
    params.push_back(LowerParam<FactorT>::run(src));
    succs.push_back(LowerSucc<SuccT, ShapeT>::run(b, src));
    StaticPairs<RestT...>::template run<ShapeT>(b, src, params, succs);
  }
};

// Subdivide<Axis, Pair<factor, successor>...>: zero factors skipped (Subdivide.cuh:22-168).
template <typename AxisT, typename... PairsT, typename ShapeT>
struct LowerOp<Operators::Subdivide<AxisT, PairsT...>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<AxisT>::run(src)};
    std::vector<PgaSuccessor> succs;
    StaticPairs<PairsT...>::template run<ShapeT>(b, src, params, succs);
    set_entry(b, i, b.proc(PGA_OP_SUBDIVIDE_STATIC, ShapeT::kind, (uint32_t)sizeof...(PairsT)), params, succs);
  }
};
// Subdivide<DynParams>: axis and factors from the entry, successor j for factor j + 1 (Subdivide.cuh:170-248).
template <typename... RestT, typename ShapeT>
struct LowerOp<Operators::Subdivide<Parameters::DynParams, RestT...>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params(src.parameters, src.parameters + src.numParameters);
    std::vector<PgaSuccessor> succs(src.successors, src.successors + src.numSuccessors);
    set_entry(b, i, b.proc(PGA_OP_SUBDIVIDE, ShapeT::kind, 0), params, succs);
  }
};
template <bool ParallelT, typename AxisT, typename ExtentT, typename ModeT, typename NextT, typename ShapeT>
struct LowerOp<Operators::Repeat<ParallelT, AxisT, ExtentT, ModeT, NextT>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<AxisT>::run(src), LowerParam<ExtentT>::run(src),
                                     LowerParam<ModeT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<NextT, ShapeT>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_REPEAT, ShapeT::kind, 0), params, succs);
  }
};
// ComponentSplit: Box -> Quads, successors (top, bottom, sides) (ComponentSplit.cuh:234-267).
template <bool ParallelT, typename TopT, typename BottomT, typename SidesT>
struct LowerOp<Operators::ComponentSplit<ParallelT, TopT, BottomT, SidesT>, Shapes::Box> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaSuccessor> succs{LowerSucc<TopT, Shapes::Quad>::run(b, src),
                                    LowerSucc<BottomT, Shapes::Quad>::run(b, src),
                                    LowerSucc<SidesT, Shapes::Quad>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_COMPONENT_SPLIT, PGA_SHAPE_BOX, 0), {}, succs);
  }
};
// Extrude: Quad -> Box (Extrude.cuh:24-69).
template <typename AxisT, typename ExtentT, typename NextT>
struct LowerOp<Operators::Extrude<AxisT, ExtentT, NextT>, Shapes::Quad> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<AxisT>::run(src), LowerParam<ExtentT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<NextT, Shapes::Box>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_EXTRUDE, PGA_SHAPE_QUAD, 0), params, succs);
  }
};
template <typename AxisT, typename SizeT, typename TrueT, typename FalseT, typename ShapeT>
struct LowerOp<Operators::IfSizeLess<AxisT, SizeT, TrueT, FalseT>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<AxisT>::run(src), LowerParam<SizeT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<TrueT, ShapeT>::run(b, src), LowerSucc<FalseT, ShapeT>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_IF_SIZE_LESS, ShapeT::kind, 0), params, succs);
  }
};
template <bool ParallelT, unsigned int GenFuncIdxT, typename TerminalIdxT, typename A1, typename A2, typename A3,
          typename A4, typename A5, typename ShapeT>
struct LowerOp<Operators::Generate<ParallelT, GenFuncIdxT, TerminalIdxT, A1, A2, A3, A4, A5>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    if (GenFuncIdxT > 1)
      throw LoweringError("generation function " + std::to_string(GenFuncIdxT) +
                          ": only 0 (triangle mesh) and 1 (instanced) are supported");
    set_entry(b, i, b.proc(GenFuncIdxT == 0 ? PGA_OP_GENERATE_MESH : PGA_OP_GENERATE, ShapeT::kind, 0),
              {LowerParam<TerminalIdxT>::run(src)}, {});
  }
};
template <typename ShapeT>
struct LowerOp<Operators::Discard, ShapeT> {
  static void run(Builder& b, const PgaEntry&, uint32_t i) {
    set_entry(b, i, b.proc(PGA_OP_DISCARD, ShapeT::kind, 0), {}, {});
  }
};
// Translate / Rotate / Scale<X, Y, Z, Next>: three parameters and the successor
// on the same shape (Translate.cuh:24-43, Rotate.cuh:24-41, Scale.cuh:23-45).
// Rotate's angles must be scalars when the engine is created.
template <uint32_t Op, typename XT, typename YT, typename ZT, typename NextT, typename ShapeT>
struct LowerXYZ {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<XT>::run(src), LowerParam<YT>::run(src), LowerParam<ZT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<NextT, ShapeT>::run(b, src)};
    set_entry(b, i, b.proc(Op, ShapeT::kind, 0), params, succs);
  }
};
template <typename XT, typename YT, typename ZT, typename NextT, typename ShapeT>
struct LowerOp<Operators::Translate<XT, YT, ZT, NextT>, ShapeT> : LowerXYZ<PGA_OP_TRANSLATE, XT, YT, ZT, NextT, ShapeT> {};
template <typename XT, typename YT, typename ZT, typename NextT, typename ShapeT>
struct LowerOp<Operators::Rotate<XT, YT, ZT, NextT>, ShapeT> : LowerXYZ<PGA_OP_ROTATE, XT, YT, ZT, NextT, ShapeT> {};
template <typename XT, typename YT, typename ZT, typename NextT, typename ShapeT>
struct LowerOp<Operators::Scale<XT, YT, ZT, NextT>, ShapeT> : LowerXYZ<PGA_OP_SCALE, XT, YT, ZT, NextT, ShapeT> {};
template <typename XT, typename YT, typename ZT, typename NextT, typename ShapeT>
struct LowerOp<Operators::SwapSize<XT, YT, ZT, NextT>, ShapeT> : LowerXYZ<PGA_OP_SWAP_SIZE, XT, YT, ZT, NextT, ShapeT> {};
// Collider<Tag, Next> (Collider.cuh:20-45) and IfCollides<Tag, True, False>
// (IfCollides.cuh:18-36); the phases of their successors come from the
// dispatch table's successor entries (PSCall / DCall keep the phase index).
template <typename TagT, typename NextT, typename ShapeT>
struct LowerOp<Operators::Collider<TagT, NextT>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<TagT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<NextT, ShapeT>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_COLLIDER, ShapeT::kind, 0), params, succs);
  }
};
template <typename TagT, typename TrueT, typename FalseT, typename ShapeT>
struct LowerOp<Operators::IfCollides<TagT, TrueT, FalseT>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<TagT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<TrueT, ShapeT>::run(b, src), LowerSucc<FalseT, ShapeT>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_IF_COLLIDES, ShapeT::kind, 0), params, succs);
  }
};
// If<Expression, True, False> (If.cuh:22-49).
template <typename ExprT, typename TrueT, typename FalseT, typename ShapeT>
struct LowerOp<Operators::If<ExprT, TrueT, FalseT>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<ExprT>::run(src)};
    std::vector<PgaSuccessor> succs{LowerSucc<TrueT, ShapeT>::run(b, src), LowerSucc<FalseT, ShapeT>::run(b, src)};
    set_entry(b, i, b.proc(PGA_OP_IF, ShapeT::kind, 0), params, succs);
  }
};
// RandomRule<DynParams>: chance and weights from the entry, successor j for weight j + 1 (RandomRule.cuh:121-150).
template <typename... RestT, typename ShapeT>
struct LowerOp<Operators::RandomRule<Parameters::DynParams, RestT...>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params(src.parameters, src.parameters + src.numParameters);
    std::vector<PgaSuccessor> succs(src.successors, src.successors + src.numSuccessors);
    set_entry(b, i, b.proc(PGA_OP_RANDOM_RULE, ShapeT::kind, 0), params, succs);
  }
};
// RandomRule<Chance, Pair<weight, successor>...>: the static form, with its own
// selection rule (RandomRule.cuh:33-99): PGA_OP_RANDOM_RULE_STATIC.
template <typename ChanceT, typename... PairsT, typename ShapeT>
struct LowerOp<Operators::RandomRule<ChanceT, PairsT...>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaParameter> params{LowerParam<ChanceT>::run(src)};
    std::vector<PgaSuccessor> succs;
    StaticPairs<PairsT...>::template run<ShapeT>(b, src, params, succs);
    set_entry(b, i, b.proc(PGA_OP_RANDOM_RULE_STATIC, ShapeT::kind, 0), params, succs);
  }
};
// Replicate<DynParams>: every successor of the entry (Replicate.cuh:95-110).
template <typename... RestT, typename ShapeT>
struct LowerOp<Operators::Replicate<Parameters::DynParams, RestT...>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaSuccessor> succs(src.successors, src.successors + src.numSuccessors);
    set_entry(b, i, b.proc(PGA_OP_REPLICATE, ShapeT::kind, 0), {}, succs);
  }
};
// Replicate<Next...>: the shape once per listed operator (Replicate.cuh:21-79).
template <typename... NextT, typename ShapeT>
struct LowerOp<Operators::Replicate<NextT...>, ShapeT> {
  static void run(Builder& b, const PgaEntry& src, uint32_t i) {
    std::vector<PgaSuccessor> succs{LowerSucc<NextT, ShapeT>::run(b, src)...};
    set_entry(b, i, b.proc(PGA_OP_REPLICATE, ShapeT::kind, 0), {}, succs);
  }
};

template <typename ProcT>
struct ProcTraits;
template <typename ShapeT, typename OperatorT, unsigned int N>
struct ProcTraits<Proc<ShapeT, OperatorT, N>> {
  static void lower(Builder& b, const PgaEntry& src, uint32_t i) { LowerOp<OperatorT, ShapeT>::run(b, src, i); }
};

template <typename... ProcsT>
T::List<ProcsT...> list_of(const T::List<ProcsT...>*);

template <typename ListT>
struct ProcList;
template <typename... ProcsT>
struct ProcList<T::List<ProcsT...>> {
  static constexpr size_t size = sizeof...(ProcsT);
  static void lower(Builder& b, size_t procIdx, const PgaEntry& src, uint32_t i) {
    using Fn = void (*)(Builder&, const PgaEntry&, uint32_t);
    static const Fn table[] = {&ProcTraits<ProcsT>::lower...};
    if (procIdx >= sizeof...(ProcsT))
      throw LoweringError("operatorCode " + std::to_string(procIdx) + " beyond the procedure list");
    table[procIdx](b, src, i);
  }
};

}  // namespace detail

/* Lowers `entries` (DispatchTableEntry layout) written for ProcedureListT, a
 * T::List<Proc<...>...> or a type derived from one, to the engine's rule table. */
template <typename ProcedureListT>
LoweredTable lower(const PgaEntry* entries, size_t numEntries) {
  using List = decltype(detail::list_of((const ProcedureListT*)nullptr));
  detail::Builder b;
  for (size_t i = 0; i < numEntries; i++) b.new_entry();
  for (size_t i = 0; i < numEntries; i++)
    detail::ProcList<List>::lower(b, entries[i].operatorCode, entries[i], (uint32_t)i);
  b.out.numUserEntries = (uint32_t)numEntries;
  return b.out;
}

template <typename ProcedureListT>
LoweredTable lower(const DispatchTable& table) {
  const std::vector<PgaEntry> e = table.toEntries();
  return lower<ProcedureListT>(e.data(), e.size());
}

}  // namespace PGA

#endif  // PGA_GB300_CORE_HPP
