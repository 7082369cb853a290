// Cell-centred heat flow, face gradient: the mean of the two cell
// gradients; a Dirichlet boundary face keeps its cell's gradient, a Neumann
// one gets the prescribed flux in every component.
{
   float4 face = 0.5f * (GrdTet[0] + GrdTet[1]);
   for(int s=0;s<6;s++)
      if(GmlPar->BoCo_Ref[s] == TriRef)
         face = GmlPar->BoCo[s] == DIRICHLET ? GrdTet[0] : (float4)(GmlPar->BoCo_Val[s]);
   GrdExt = face;
}
