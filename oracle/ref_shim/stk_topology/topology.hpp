// Stand-in for stk::topology with the hex8 side queries the SCS constructor uses.
#pragma once
namespace stk {
struct topology {
  enum topology_t { INVALID_TOPOLOGY, QUAD_4, HEX_8, HEXAHEDRON_8 = HEX_8, HEX_27, TET_4, PYRAMID_5,
                    WEDGE_6, QUAD_4_2D, QUAD_9_2D, TRI_3_2D, TRI_3, QUAD_9, TRI_6, TET_10, SHELL_QUAD_4,
                    LINE_2, LINE_3, QUAD_8_2D, TRI_6_2D, BEAM_2, BEAM_3, SHELL_TRI_3, SHELL_QUAD_9, PARTICLE, WEDGE_15, WEDGE_18, HEX_20, PYRAMID_13, PYRAMID_14, TET_8, TET_11, QUAD_8, TRI_4, LINE_2_1D, LINE_3_1D, SPRING_2, SPRING_3 };
  topology_t t;
  topology(topology_t v = INVALID_TOPOLOGY) : t(v) {}
  operator topology_t() const { return t; }
  unsigned num_sides() const { return t == HEX_8 ? 6 : 0; }
  topology side_topology(unsigned) const { return t == HEX_8 ? QUAD_4 : INVALID_TOPOLOGY; }
  unsigned num_nodes() const { return t == HEX_8 ? 8 : (t == QUAD_4 ? 4 : 0); }
};
}
