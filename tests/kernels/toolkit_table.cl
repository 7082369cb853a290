// Every function of the geometric toolkit on one point set Pts[0..7] (a
// jittered hexahedron in the GMlib corner order), 60 results in Res.
// Compiled by GmlCompileKernel on the GPU and, by oracle/refcl, against the
// reference's own sources/toolkit.cl on the CPU.
{
   float4 a = Pts[0], b = Pts[1], c = Pts[2], d = Pts[3];
   float4 e = Pts[4], f = Pts[5], g = Pts[6], h = Pts[7];
   float4 t, u, v;
   float16 m;
   int i = 0;

   Res[i++] = DisPow(a, g);
   Res[i++] = CalLen(a, g);
   Res[i++] = CalSrf(a, b, d);
   Res[i++] = CalVol(a, b, d, e);
   Res[i++] = CalEdgLen(b, h);
   Res[i++] = CalTriSrf(a, c, f);
   Res[i++] = CalQadSrf(a, b, c, d);
   Res[i++] = CalTetVol(a, b, d, e);
   Res[i++] = CalPyrVol(a, b, c, d, g);
   Res[i++] = CalPriVol(a, b, d, e, f, h);
   Res[i++] = CalHexVol(a, b, c, d, e, f, g, h);
   Res[i++] = CalTriQal(a, c, f);
   Res[i++] = CalQadQal(a, b, c, d);
   Res[i++] = CalTetQal(a, b, d, e);
   Res[i++] = CalPyrQal(a, b, c, d, g);
   Res[i++] = CalPriQal(a, b, d, e, f, h);
   Res[i++] = CalHexQal(a, b, c, d, e, f, g, h);
   Res[i++] = DisVerLin(g, a, GetEdgTng(a, b));
   Res[i++] = DisVerPla(g, a, GetTriNrm(a, b, d));
   Res[i++] = DisVerEdg(g, a, b, GetEdgTng(a, b));

   t = GetEdgTng(a, g);
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   t = GetTriNrm(a, b, d);
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   t = GetQadNrm(a, b, c, d);
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   t = PrjVerLin(g, a, GetEdgTng(a, b));
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   t = PrjVerPla(g, a, GetTriNrm(a, b, d));
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   t = LinIntLin(a, GetEdgTng(a, g), b, GetEdgTng(b, h));
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   t = LinIntPla(a, GetEdgTng(a, g), e, GetTriNrm(e, f, h));
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;
   PlaIntPla(a, GetTriNrm(a, b, d), a, GetTriNrm(a, e, b), &u, &v);
   Res[i++] = u.x; Res[i++] = u.y; Res[i++] = u.z; Res[i++] = u.w;
   Res[i++] = v.x; Res[i++] = v.y; Res[i++] = v.z; Res[i++] = v.w;
   m.s0 = a.x; m.s1 = a.y; m.s2 = a.z; m.s3 = b.x;
   m.s4 = b.y; m.s5 = b.z; m.s6 = c.x; m.s7 = c.y;
   m.s8 = c.z; m.s9 = d.x; m.sa = d.y; m.sb = d.z;
   m.sc = e.x; m.sd = e.y; m.se = e.z; m.sf = f.x;
   t = MulMatVec(m, g);
   Res[i++] = t.x; Res[i++] = t.y; Res[i++] = t.z; Res[i++] = t.w;

   while(i < 64)
      Res[i++] = 0.f;
}
