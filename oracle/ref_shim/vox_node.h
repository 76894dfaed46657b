// vox_node.h - the VoxNode layout of reaction/report/main.tex:36-56 (the
// reference's header is not in its snapshot): flags bits 0-7 leaf, 8-15
// null; child ids with bit 31 set are null (EmptyNode / FullNode).
#pragma once
#include <cstdint>

typedef unsigned int uint;
typedef uint VoxNodeId;
typedef uint VoxData;

const VoxNodeId EmptyNode = 0x80000000u;
const VoxNodeId FullNode = 0x80000001u;

struct VoxNode {
  uint flags;
  VoxData data;
  VoxNodeId child[8];
};

inline bool IsNull(VoxNodeId id) { return (id & 0x80000000u) != 0; }
inline bool GetLeafFlag(uint flags, int ch) { return ((flags >> ch) & 1u) != 0; }
