// Grammars written with the C++ operator API (pga/core.hpp) in the reference's
// own syntax, lowered to rule tables and written to a file for the Python
// tests, which derive them with the oracle and compare with the same grammars
// built as data (operatorgraph_gb300/scenes.py).
//
// Output: per scene  u32 nameLen, name, u32 numProcs, PgaProc[], u32 numEntries,
// PgaEntry[], u32 numUserEntries.  A lowering that throws writes numProcs =
// 0xFFFFFFFF and the message instead.
#include <pga/core.hpp>

#include <cstdio>
#include <string>

using namespace PGA;
using namespace PGA::Operators;
using namespace PGA::Parameters;
using namespace PGA::Shapes;

namespace menger {
// Procedure list of the reference's test-runner Menger scene
// (src/test_runner/MengerSponge.cuh:28-33): everything from the table.
struct ProcedureList
    : T::List<Proc<Box, Subdivide<DynParam<0>, T::Pair<DynParam<1>, DCall<0>>, T::Pair<DynParam<2>, DCall<1>>,
                                  T::Pair<DynParam<3>, DCall<2>>>, 1>,
              Proc<Box, Discard, 1>,
              Proc<Box, IfSizeLess<DynParam<0>, DynParam<1>, DCall<0>, DCall<1>>, 1>,
              Proc<Box, Generate<false, 1, DynParam<0>>, 1>> {};

// Entry 0 tests the size against the threshold, entry 2..5,7 split along X, Y,
// Z into thirds with the centre pieces discarded (the same table as
// scenes.menger_table(0.05)).
DispatchTable table() {
  using P = DispatchTable::Parameter;
  const P rel{PT_SCALAR, {-1}};
  return DispatchTable{
      {2, {P{PT_SCALAR, {0}}, P{PT_SCALAR, {0.05}}}, {{1, 0}, {2, 0}}},
      {3, {P{PT_SCALAR, {0}}}, {}},
      {0, {P{PT_SCALAR, {0}}, rel, rel, rel}, {{3, 0}, {7, 0}, {3, 0}}},
      {0, {P{PT_SCALAR, {1}}, rel, rel, rel}, {{4, 0}, {5, 0}, {4, 0}}},
      {0, {P{PT_SCALAR, {2}}, rel, rel, rel}, {{0, 0}, {0, 0}, {0, 0}}},
      {0, {P{PT_SCALAR, {2}}, rel, rel, rel}, {{0, 0}, {6, 0}, {0, 0}}},
      {1, {}, {}},
      {0, {P{PT_SCALAR, {1}}, rel, rel, rel}, {{5, 0}, {8, 0}, {5, 0}}},
      {1, {}, {}},
  };
}
}  // namespace menger

namespace building_dyn {
// The one-building grammar with every argument dynamic (one procedure per operator and shape).
struct ProcedureList
    : T::List<Proc<Quad, Extrude<DynParam<0>, DynParam<1>, DCall<0>>, 1>,
              Proc<Box, ComponentSplit<false, DCall<0>, DCall<1>, DCall<2>>, 1>,
              Proc<Quad, Repeat<false, DynParam<0>, DynParam<1>, DynParam<2>, DCall<0>>, 1>,
              Proc<Quad, IfSizeLess<DynParam<0>, DynParam<1>, DCall<0>, DCall<1>>, 1>,
              Proc<Quad, Subdivide<DynParams>, 1>,
              Proc<Quad, Generate<false, 1, DynParam<0>>, 1>,
              Proc<Quad, Discard, 1>> {};

DispatchTable table(int mode) {
  using P = DispatchTable::Parameter;
  return DispatchTable{
      {0, {P{PT_SCALAR, {1}}, P{PT_SHAPE_ATTR, {16}}}, {{1, 0}}},
      {1, {}, {{9, 0}, {7, 0}, {2, 0}}},
      {2, {P{PT_SCALAR, {1}}, P{PT_SCALAR, {3.0}}, P{PT_SCALAR, {(double)mode}}}, {{3, 0}}},
      {2, {P{PT_SCALAR, {0}}, P{PT_SCALAR, {2.5}}, P{PT_SCALAR, {(double)mode}}}, {{4, 0}}},
      {3, {P{PT_SCALAR, {0}}, P{PT_SCALAR, {1.2}}}, {{7, 0}, {5, 0}}},
      {4, {P{PT_SCALAR, {0}}, P{PT_SCALAR, {0.2}}, P{PT_SCALAR, {-1}}, P{PT_SCALAR, {0.2}}}, {{8, 0}, {6, 0}, {8, 0}}},
      {5, {P{PT_SCALAR, {1}}}, {}},
      {6, {}, {}},
      {5, {P{PT_SCALAR, {0}}}, {}},
      {5, {P{PT_SCALAR, {2}}}, {}},
  };
}
}  // namespace building_dyn

namespace building_static {
// The same building as ONE procedure whose operators are chained statically,
// with static parameters: Extrude to the custom-attribute height, split off
// roof (terminal 2) and bottom (discarded), floors of 3 m, tiles of 2.5 m,
// narrow tiles discarded, others split into wall / window / wall.
template <RepeatMode M>
using Tile = IfSizeLess<AxisParam<X>, Scalar<12, 1>, Discard,
                        Subdivide<AxisParam<X>, T::Pair<Scalar<2, 1>, Generate<false, 1, Scalar<0>>>,
                                  T::Pair<Scalar<-1>, Generate<false, 1, Scalar<1>>>,
                                  T::Pair<Scalar<2, 1>, Generate<false, 1, Scalar<0>>>>>;
template <RepeatMode M>
using Facade = Repeat<false, AxisParam<Y>, Scalar<3>, RepeatModeParam<M>,
                      Repeat<false, AxisParam<X>, Scalar<25, 1>, RepeatModeParam<M>, Tile<M>>>;
template <RepeatMode M>
struct ProcedureList
    : T::List<Proc<Quad,
                   Extrude<AxisParam<Y>, ShapeCustomAttribute,
                           ComponentSplit<false, Generate<false, 1, Scalar<2>>, Discard, Facade<M>>>,
                   1>> {};

DispatchTable table() { return DispatchTable{{0, {}, {}}}; }
}  // namespace building_static

namespace building_exp {
// The static building again, with parameters given as expressions that
// evaluate to the same values: 3 = 1.5 * 2, 2.5 = 5 / 2, 1.2 = 12 / 10 and the
// window share -1 = 0 - 1.
using Tile = IfSizeLess<AxisParam<X>, Exp<Scalar<12>, Scalar<10>, Div>, Discard,
                        Subdivide<AxisParam<X>, T::Pair<Scalar<2, 1>, Generate<false, 1, Scalar<0>>>,
                                  T::Pair<Exp<Scalar<0>, Scalar<1>, Sub>, Generate<false, 1, Scalar<1>>>,
                                  T::Pair<Scalar<2, 1>, Generate<false, 1, Scalar<0>>>>>;
using Facade = Repeat<false, AxisParam<Y>, Exp<Scalar<15, 1>, Scalar<2>, Multi>, RepeatModeParam<ANCHOR_TO_START>,
                      Repeat<false, AxisParam<X>, Exp<Scalar<5>, Scalar<2>, Div>, RepeatModeParam<ANCHOR_TO_START>,
                             Tile>>;
struct ProcedureList
    : T::List<Proc<Quad,
                   Extrude<AxisParam<Y>, ShapeCustomAttribute,
                           ComponentSplit<false, Generate<false, 1, Scalar<2>>, Discard, Facade>>,
                   1>> {};
}  // namespace building_exp

namespace calls {
// Successor kinds: PSCall and FSCall next to DCall (Call.cuh:23-260): the
// Menger table reached through partially and fully static calls.
struct ProcedureList
    : T::List<Proc<Box, Subdivide<DynParam<0>, T::Pair<DynParam<1>, PSCall<0, 0>>, T::Pair<DynParam<2>, DCall<1>>,
                                  T::Pair<DynParam<3>, PSCall<0, 2>>>, 1>,
              Proc<Box, Discard, 1>,
              Proc<Box, IfSizeLess<DynParam<0>, DynParam<1>, FSCall<3, 0, -1, 1>, DCall<1>>, 1>,
              Proc<Box, Generate<false, 1, DynParam<0>>, 1>> {};
}  // namespace calls

namespace random_static_dyn {
// The static RandomRule with DynParam weights and DCall successors (2, 3 and 4
// pairs, both shapes) plus ComponentSplit / Generate / Discard: the same
// grammar as tests/golden/cases.py random_static_mix, procedure for procedure.
template <typename ShapeT, typename... PairsT>
using RR = Proc<ShapeT, RandomRule<DynParam<0>, PairsT...>, 1>;
using P1 = T::Pair<DynParam<1>, DCall<0>>;
using P2 = T::Pair<DynParam<2>, DCall<1>>;
using P3 = T::Pair<DynParam<3>, DCall<2>>;
using P4 = T::Pair<DynParam<4>, DCall<3>>;
struct ProcedureList
    : T::List<RR<Box, P1, P2, P3>,                                            // 0
              Proc<Box, Generate<false, 1, DynParam<0>>, 1>,                  // 1
              Proc<Box, ComponentSplit<false, DCall<0>, DCall<1>, DCall<2>>, 1>,  // 2
              RR<Box, P1, P2, P3, P4>,                                        // 3
              RR<Quad, P1, P2>,                                               // 4
              Proc<Quad, Discard, 1>,                                         // 5
              RR<Quad, P1, P2, P3>,                                           // 6
              Proc<Quad, Generate<false, 1, DynParam<0>>, 1>,                 // 7
              RR<Quad, P1, P2, P3, P4>> {};                                   // 8

DispatchTable table() {
  using P = DispatchTable::Parameter;
  auto s = [](double v) { return P{PT_SCALAR, {v}}; };
  const P seed{PT_SHAPE_ATTR, {15}}, custom{PT_SHAPE_ATTR, {16}}, rnd{PT_RAND, {0.0, 1.0}};
  return DispatchTable{
      {0, {seed, s(0.333), s(0.333), s(0.333)}, {{1, 0}, {2, 0}, {3, 0}}},
      {1, {s(0)}, {}},
      {2, {}, {{4, 0}, {5, 0}, {6, 0}}},
      {3, {custom, s(0.1), s(0.2), s(0.3), s(0.15)}, {{1, 0}, {7, 0}, {8, 0}, {9, 0}}},
      {4, {seed, s(0.0), s(1.0)}, {{10, 0}, {11, 0}}},
      {5, {}, {}},
      {6, {rnd, s(2.0), s(0.0), s(1.0)}, {{10, 0}, {11, 0}, {12, 0}}},
      {1, {s(1)}, {}},
      {1, {s(2)}, {}},
      {1, {s(3)}, {}},
      {7, {s(4)}, {}},
      {7, {s(5)}, {}},
      {8, {custom, s(0.25), s(0.25), s(0.25), s(0.25)}, {{10, 0}, {11, 0}, {13, 0}, {11, 0}}},
      {7, {s(6)}, {}},
  };
}
}  // namespace random_static_dyn

namespace rotate_static {
// One procedure, statically chained: a box replicated into an unrotated
// copy, a copy turned 90 degrees about y then split along x (the second piece
// turned -37 degrees about z), and a copy turned (30, -47.5, 12.25) degrees
// then split into faces; the top face turned 45 degrees, translated by
// (0.5, size_y / 2, -0.25), scaled to (x / 2, 2, 1) and extruded to 0.75; the
// sides replicated into the face itself and a copy turned (90, 90, 0).
using Gen0 = Generate<false, 1, Scalar<0>>;
using QGen1 = Generate<false, 1, Scalar<1>>;
using Turned = Rotate<Scalar<0>, Scalar<0>, Scalar<-37>, Gen0>;
using Top = Rotate<Scalar<0>, Scalar<0>, Scalar<45>,
                   Translate<Scalar<5, 1>, Exp<ShapeSize<Y>, Scalar<5, 1>, Multi>, Scalar<-25, 2>,
                             Scale<Scalar<-5, 1>, Scalar<2>, Scalar<1>, Extrude<AxisParam<X>, Scalar<75, 2>, Gen0>>>>;
using Sides = Replicate<QGen1, Rotate<Scalar<90>, Scalar<90>, Scalar<0>, QGen1>>;
struct ProcedureList
    : T::List<Proc<Box,
                   Replicate<Gen0,
                             Rotate<Scalar<0>, Scalar<90>, Scalar<0>,
                                    Subdivide<AxisParam<X>, T::Pair<Scalar<-1>, Gen0>, T::Pair<Scalar<-2>, Turned>>>,
                             Rotate<Scalar<30>, Scalar<-475, 1>, Scalar<1225, 2>,
                                    ComponentSplit<false, Top, Discard, Sides>>>,
                   1>> {};
}  // namespace rotate_static

namespace if_swap_static {
// If on an expression (size x > 1.5): the sizes cycled (y, z, x) then a box
// terminal; otherwise split along x into a terminal and a piece whose sizes
// are swapped (x, z, y) before it becomes a terminal of index 1.
using Gen0 = Generate<false, 1, Scalar<0>>;
using Gen1 = Generate<false, 1, Scalar<1>>;
struct ProcedureList
    : T::List<Proc<Box,
                   If<Exp<ShapeSize<X>, Scalar<15, 1>, Gt>, SwapSize<AxisParam<Y>, AxisParam<Z>, AxisParam<X>, Gen0>,
                      Subdivide<AxisParam<X>, T::Pair<Scalar<-1>, Gen0>,
                                T::Pair<Scalar<-1>, SwapSize<AxisParam<X>, AxisParam<Z>, AxisParam<Y>, Gen1>>>>,
                   1>> {};
}  // namespace if_swap_static

namespace bad {
// A generation function other than 0 (triangle mesh) and 1 (instanced).
struct ProcedureList : T::List<Proc<Box, Generate<false, 2, Scalar<0>>, 1>> {};
}  // namespace bad

namespace mesh_terminals {
// Triangle-mesh terminals (GenFuncIdx 0) beside instanced ones: a box split
// into faces; the top is a mesh quad, the sides instanced, the box itself a
// mesh box.
struct ProcedureList
    : T::List<Proc<Box,
                   Replicate<Generate<false, 0, Scalar<0>>,
                             ComponentSplit<false, Generate<false, 0, Scalar<1>>, Discard, Generate<false, 1, Scalar<2>>>>,
                   1>> {};
}  // namespace mesh_terminals

static void write_scene(FILE* f, const std::string& name, const LoweredTable& t) {
  const uint32_t n = (uint32_t)name.size();
  fwrite(&n, 4, 1, f);
  fwrite(name.data(), 1, n, f);
  const uint32_t np = (uint32_t)t.procs.size(), ne = (uint32_t)t.entries.size();
  fwrite(&np, 4, 1, f);
  fwrite(t.procs.data(), sizeof(PgaProc), np, f);
  fwrite(&ne, 4, 1, f);
  fwrite(t.entries.data(), sizeof(PgaEntry), ne, f);
  fwrite(&t.numUserEntries, 4, 1, f);
}

static void write_error(FILE* f, const std::string& name, const std::string& msg) {
  const uint32_t n = (uint32_t)name.size(), bad = 0xFFFFFFFFu, m = (uint32_t)msg.size();
  fwrite(&n, 4, 1, f);
  fwrite(name.data(), 1, n, f);
  fwrite(&bad, 4, 1, f);
  fwrite(&m, 4, 1, f);
  fwrite(msg.data(), 1, m, f);
}

template <typename ListT>
static void scene(FILE* f, const std::string& name, const DispatchTable& table) {
  try {
    write_scene(f, name, lower<ListT>(table));
  } catch (const std::exception& e) {
    write_error(f, name, e.what());
  }
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s out.bin\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  scene<menger::ProcedureList>(f, "menger", menger::table());
  for (int mode = 0; mode < 3; mode++)
    scene<building_dyn::ProcedureList>(f, "building_dyn_m" + std::to_string(mode), building_dyn::table(mode));
  scene<building_static::ProcedureList<ANCHOR_TO_START>>(f, "building_static_m0", building_static::table());
  scene<building_static::ProcedureList<ANCHOR_TO_END>>(f, "building_static_m1", building_static::table());
  scene<building_static::ProcedureList<ADJUST_TO_FILL>>(f, "building_static_m2", building_static::table());
  scene<building_exp::ProcedureList>(f, "building_exp", building_static::table());
  scene<calls::ProcedureList>(f, "menger_calls", menger::table());
  scene<random_static_dyn::ProcedureList>(f, "random_static_dyn", random_static_dyn::table());
  scene<rotate_static::ProcedureList>(f, "rotate_static", building_static::table());
  scene<if_swap_static::ProcedureList>(f, "if_swap_static", building_static::table());
  scene<bad::ProcedureList>(f, "bad_generation_function", DispatchTable{{0, {}, {}}});
  scene<mesh_terminals::ProcedureList>(f, "mesh_terminals", DispatchTable{{0, {}, {}}});
  scene<menger::ProcedureList>(f, "bad_dynparam", DispatchTable{{2, {}, {{1, 0}, {2, 0}}}});
  std::fclose(f);
  return 0;
}
