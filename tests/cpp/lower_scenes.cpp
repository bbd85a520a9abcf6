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

namespace bad {
// Triangle-mesh generation (GenFuncIdx 0) is outside the engine.
struct ProcedureList : T::List<Proc<Box, Generate<false, 0, Scalar<0>>, 1>> {};
}  // namespace bad

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
  scene<bad::ProcedureList>(f, "triangle_mesh", DispatchTable{{0, {}, {}}});
  scene<menger::ProcedureList>(f, "bad_dynparam", DispatchTable{{2, {}, {{1, 0}, {2, 0}}}});
  std::fclose(f);
  return 0;
}
