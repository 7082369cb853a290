// Cell-centred heat flow, face value: the mean of the cells on either side
// of the face; a boundary face (reference TriRef) under a Dirichlet
// condition takes the prescribed value, under a Neumann condition the value
// of its single cell.
{
   float face = 0.5f * (SolTet[0] + SolTet[1]);
   for(int s=0;s<6;s++)
      if(GmlPar->BoCo_Ref[s] == TriRef)
         face = GmlPar->BoCo[s] == DIRICHLET ? GmlPar->BoCo_Val[s] : SolTet[0];
   SolExt = face;
}
