// Cell-centred heat flow, flux balance: the sum over the four faces of face
// gradient dotted with the area vector, divided by the volume.
{
   const int fv[4][3] = { {1, 2, 3}, {2, 0, 3}, {3, 0, 1}, {0, 2, 1} };
   float r = 0.f;
   for(int j=0;j<4;j++)
      r += dot(GrdExt[j], cross(VerCrd[ fv[j][1] ] - VerCrd[ fv[j][0] ],
                                VerCrd[ fv[j][2] ] - VerCrd[ fv[j][0] ]));
   Rhs = 0.5f * r / CalTetVol(VerCrd[0], VerCrd[1], VerCrd[2], VerCrd[3]);
}
