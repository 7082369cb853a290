// Which tets a triangle's shell lists, in which order: a tet field holding
// index + 1, read through the triangle -> tet uplink (0 past the degree).
{
   ShlTet.x = TetNum[0];
   ShlTet.y = TetNum[1];
   ShlTet.z = (float)TetNumDeg;
   ShlTet.w = 0.f;
}
