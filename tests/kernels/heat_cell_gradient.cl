// Cell-centred heat flow, cell gradient: Green-Gauss sum over the four
// faces (face j opposite vertex j, its area vector from the table below)
// of face value times area vector, divided by the volume.
{
   const int fv[4][3] = { {1, 2, 3}, {2, 0, 3}, {3, 0, 1}, {0, 2, 1} };
   float4 g = (float4)(0.f);
   for(int j=0;j<4;j++)
      g += SolExt[j] * cross(VerCrd[ fv[j][1] ] - VerCrd[ fv[j][0] ],
                             VerCrd[ fv[j][2] ] - VerCrd[ fv[j][0] ]);
   GrdTet = 0.5f * g / CalTetVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]);
}
