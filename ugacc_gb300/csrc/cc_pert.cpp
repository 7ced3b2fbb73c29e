// Perturbed wavefunctions (ccpert.cc:11-881) and linear response (ccresp.cc:28-124).
//
// The left-hand residual of the reference (build_Y1/build_Y2) contains products of an
// amplitude, an HBAR or integral block and a Lambda amplitude summed over up to six
// indices (O(no^4 nv^4) as written, ccpert.cc:689-699, :834-872).  Each such product is
// evaluated here as two pairwise contractions through a small intermediate.
#include <cmath>
#include <cstdio>

#include "pert.h"

namespace ucc {

namespace {
void copy_into(Ctx& c, const Tensor& src, Tensor dst) { permute_add(c, src, 1.0, 0.0, dst); }

Perturbation& get_pert(Ctx& c, int h) {
  UCC_REQUIRE(h >= 0 && h < (int)c.perts.size(), UCC_BAD_ARGS, "bad perturbation handle");
  return *c.perts[h];
}
Tensor P(Ctx& c, const Perturbation& p, const char* nm) { return c.get(p.pfx + nm); }

// pertbar, ccpert.cc:109-175
void pertbar(Ctx& c, Perturbation& p) {
  const int no = c.no, nv = c.nv;
  double* T = c.get("T").p;
  Tensor t1 = amp1(c, T), t2 = amp2(c, T);
  Tensor pov = P(c, p, "pov"), poo = P(c, p, "poo"), pvv = P(c, p, "pvv"), pvo = P(c, p, "pvo");
  Tensor Aoo = c.alloc(p.pfx + "Aoo", {no, no}, false);
  copy_into(c, poo, Aoo);
  contract(c, "ie,me->mi", 1.0, t1, pov, 1.0, Aoo);
  Tensor Avv = c.alloc(p.pfx + "Avv", {nv, nv}, false);
  copy_into(c, pvv, Avv);
  contract(c, "ma,me->ae", -1.0, t1, pov, 1.0, Avv);
  Tensor Avo = c.alloc(p.pfx + "Avo", {nv, no}, false);
  copy_into(c, pvo, Avo);
  contract(c, "ie,ae->ai", 1.0, t1, pvv, 1.0, Avo);
  contract(c, "ma,mi->ai", -1.0, t1, poo, 1.0, Avo);
  {
    Temp X(c, {no, no, nv, nv});  // 2 t2[m,i,e,a] - t2[i,m,e,a]
    transpose_add(c, "imea->miea", -1.0, t2, 0.0, X);
    axpby(c, X->size(), 2.0, t2.p, 1.0, X->p);
    contract(c, "miea,me->ai", 1.0, X, pov, 1.0, Avo);
    Temp Y(c, {no, no});  // Y[i,m] = t1[i,e] pov[m,e]
    contract(c, "ie,me->im", 1.0, t1, pov, 0.0, Y);
    contract(c, "im,ma->ai", -1.0, Y, t1, 1.0, Avo);
  }
  Tensor Aovoo = c.alloc(p.pfx + "Aovoo", {no, nv, no, no}, false);
  contract(c, "ijeb,me->mbij", 1.0, t2, pov, 0.0, Aovoo);
  Tensor Avvvo = c.alloc(p.pfx + "Avvvo", {nv, nv, nv, no}, false);
  contract(c, "miab,me->abei", -1.0, t2, pov, 0.0, Avvvo);
  Tensor Avvoo = c.alloc(p.pfx + "Avvoo", {nv, nv, no, no}, false);
  contract(c, "ijeb,ae->abij", 1.0, t2, Avv, 0.0, Avvoo);
  contract(c, "mjab,mi->abij", -1.0, t2, Aoo, 1.0, Avvoo);
}

// build_X1 / build_X2, ccpert.cc:373-473
void build_X(Ctx& c, Perturbation& p, const Tensor& X1o, const Tensor& X2o, Tensor R1, Tensor R2) {
  const int no = c.no, nv = c.nv;
  const double w = p.omega;
  Tensor t2 = amp2(c, c.get("T").p);
  transpose_add(c, "ai->ia", 1.0, P(c, p, "Avo"), 0.0, R1);
  axpby(c, R1.size(), -w, X1o.p, 1.0, R1.p);
  contract(c, "ie,ae->ia", 1.0, X1o, c.get("Hvv"), 1.0, R1);
  contract(c, "ma,mi->ia", -1.0, X1o, c.get("Hoo"), 1.0, R1);
  contract(c, "me,maei->ia", 1.0, X1o, c.get("Hovvo_x"), 1.0, R1);  // 2 Hovvo[m,a,e,i] - Hovov[m,a,i,e]
  {
    Temp X(c, {no, no, nv, nv});  // 2 X2[m,i,e,a] - X2[i,m,e,a]
    transpose_add(c, "imea->miea", -1.0, X2o, 0.0, X);
    axpby(c, X->size(), 2.0, X2o.p, 1.0, X->p);
    contract(c, "me,miea->ia", 1.0, c.get("Hov"), X, 1.0, R1);
  }
  // 2 Hvovv[a,m,e,f] - Hvovv[a,m,f,e] = Hvovv_x[a,m,e,f]
  Tensor Hvovv_xs = c.get("Hvovv_x");
  contract(c, "imef,amef->ia", 1.0, X2o, Hvovv_xs, 1.0, R1);
  // 2 Hooov[m,n,i,e] - Hooov[n,m,i,e] = Hooov_x[m,n,i,e]
  contract(c, "mnae,mnie->ia", -1.0, X2o, c.get("Hooov_x"), 1.0, R1);

  Tensor Lv = L(c, "oovv");
  Temp Zvv(c, {nv, nv}), Zoo(c, {no, no});
  contract(c, "amef,mf->ae", 1.0, Hvovv_xs, X1o, 0.0, Zvv);
  contract(c, "mnef,mnaf->ae", -1.0, Lv, X2o, 1.0, Zvv);
  contract(c, "mnie,ne->mi", -1.0, c.get("Hooov_x"), X1o, 0.0, Zoo);
  contract(c, "mnef,inef->mi", -1.0, Lv, X2o, 1.0, Zoo);

  Temp Q(c, {no, no, nv, nv});
  transpose_add(c, "abij->ijab", 1.0, P(c, p, "Avvoo"), 0.0, Q);
  axpby(c, Q->size(), -0.5 * w, X2o.p, 1.0, Q->p);
  contract(c, "ie,abej->ijab", 1.0, X1o, c.get("Hvvvo"), 1.0, Q);
  contract(c, "ma,mbij->ijab", -1.0, X1o, c.get("Hovoo"), 1.0, Q);
  contract(c, "mi,mjab->ijab", 1.0, Zoo, t2, 1.0, Q);
  contract(c, "ae,ijeb->ijab", 1.0, Zvv, t2, 1.0, Q);
  contract(c, "ijeb,ae->ijab", 1.0, X2o, c.get("Hvv"), 1.0, Q);
  contract(c, "mjab,mi->ijab", -1.0, X2o, c.get("Hoo"), 1.0, Q);
  contract(c, "mnab,mnij->ijab", 0.5, X2o, c.get("Hoooo"), 1.0, Q);
  // 0.5 sum_ef X2_ijef Hvvvv_abef, moved past the symmetrisation: W_abef = Hvvvv_abef + Hvvvv_bafe
  const bool packed = hbar_ladder_packed(c);
  if (!packed) contract(c, "ijef,abef->ijab", 0.5, X2o, c.get("Hvvvv"), 1.0, Q);
  contract(c, "imeb,maje->ijab", -1.0, X2o, c.get("Hovov"), 1.0, Q);
  contract(c, "imea,mbej->ijab", -1.0, X2o, c.get("Hovvo"), 1.0, Q);
  contract(c, "miea,mbej->ijab", 1.0, X2o, c.get("Hovvo_x"), 1.0, Q);  // 2 Hovvo[m,b,e,j] - Hovov[m,b,j,e]
  copy_into(c, Q, R2);
  transpose_add(c, "jiba->ijab", 1.0, Q, 1.0, R2);
  if (packed) packed_ladder(c, 0.5, X2o, "Hvvvv", 2, "Hpp2", "Hmm2", R2.p);
}

// build_G / build_Y1 / build_Y2, ccpert.cc:500-881
void build_Y(Ctx& c, Perturbation& p, const Tensor& Y1o, const Tensor& Y2o, Tensor R1, Tensor R2) {
  const int no = c.no, nv = c.nv;
  const double w = p.omega;
  Tensor t2 = amp2(c, c.get("T").p);
  double* Lp = c.get("Lam").p;
  Tensor l1 = amp1(c, Lp), l2 = amp2(c, Lp);
  double* Xp = c.get(p.pfx + "X").p;
  Tensor X1 = amp1(c, Xp), X2 = amp2(c, Xp);
  Tensor Hov = c.get("Hov"), Hoo = c.get("Hoo"), Hvv = c.get("Hvv"), Hoooo = c.get("Hoooo"), Hvvvv = c.get("Hvvvv");
  Tensor Hovvo = c.get("Hovvo"), Hovov = c.get("Hovov"), Hvovv = c.get("Hvovv"), Hooov = c.get("Hooov");
  Tensor Hvvvo = c.get("Hvvvo"), Hovoo = c.get("Hovoo");
  Tensor Hovvo_x = c.get("Hovvo_x"), Hvovv_x = c.get("Hvovv_x"), Hooov_x = c.get("Hooov_x");
  Tensor Lv = L(c, "oovv"), Vv = V(c, "oovv");
  Tensor Aoo = P(c, p, "Aoo"), Avv = P(c, p, "Avv"), Avvvo = P(c, p, "Avvvo"), Aovoo = P(c, p, "Aovoo");
  Tensor pov = P(c, p, "pov");

  Temp Goo(c, {no, no}), Gvv(c, {nv, nv});
  contract(c, "mjab,ijab->mi", 1.0, t2, Y2o, 0.0, Goo);
  contract(c, "ijeb,ijab->ae", -1.0, t2, Y2o, 0.0, Gvv);

  // ---------------- Y1 ----------------
  axpby(c, R1.size(), 2.0, pov.p, 0.0, R1.p);
  axpby(c, R1.size(), w, Y1o.p, 1.0, R1.p);
  contract(c, "ie,ea->ia", 1.0, Y1o, Hvv, 1.0, R1);
  contract(c, "ma,im->ia", -1.0, Y1o, Hoo, 1.0, R1);
  contract(c, "me,ieam->ia", 1.0, Y1o, Hovvo_x, 1.0, R1);
  contract(c, "imef,efam->ia", 1.0, Y2o, Hvvvo, 1.0, R1);
  contract(c, "mnae,iemn->ia", -1.0, Y2o, Hovoo, 1.0, R1);
  contract(c, "ef,eifa->ia", -1.0, Gvv, Hvovv_x, 1.0, R1);
  contract(c, "mn,mina->ia", -1.0, Goo, Hooov_x, 1.0, R1);
  contract(c, "me,imae->ia", 2.0, X1, Lv, 1.0, R1);                     // (i)
  contract(c, "ma,im->ia", -1.0, l1, Aoo, 1.0, R1);                     // (m)
  contract(c, "ie,ea->ia", 1.0, l1, Avv, 1.0, R1);
  contract(c, "imfe,feam->ia", 1.0, l2, Avvvo, 1.0, R1);                // (n)
  contract(c, "mnea,ienm->ia", -0.5, l2, Aovoo, 1.0, R1);
  contract(c, "mnae,iemn->ia", -0.5, l2, Aovoo, 1.0, R1);
  {  // (q)
    Temp Pae(c, {nv, nv}), Qmi(c, {no, no}), Smn(c, {no, no}), Tin(c, {no, no}), Ufa(c, {nv, nv}), Wef(c, {nv, nv});
    contract(c, "me,ma->ae", 1.0, X1, Hov, 0.0, Pae);
    contract(c, "ae,ie->ia", -1.0, Pae, l1, 1.0, R1);
    contract(c, "me,ie->mi", 1.0, X1, Hov, 0.0, Qmi);
    contract(c, "mi,ma->ia", -1.0, Qmi, l1, 1.0, R1);
    contract(c, "me,ne->mn", 1.0, X1, l1, 0.0, Smn);
    contract(c, "mn,mina->ia", -1.0, Smn, Hooov_x, 1.0, R1);
    contract(c, "me,imne->in", 1.0, X1, Hooov_x, 0.0, Tin);
    contract(c, "in,na->ia", -1.0, Tin, l1, 1.0, R1);
    contract(c, "me,fmae->fa", 1.0, X1, Hvovv_x, 0.0, Ufa);
    contract(c, "fa,if->ia", 1.0, Ufa, l1, 1.0, R1);
    contract(c, "me,mf->ef", 1.0, X1, l1, 0.0, Wef);
    contract(c, "ef,fiea->ia", 1.0, Wef, Hvovv_x, 1.0, R1);
  }
  {  // (r)
    Temp Z1(c, {no, nv}), Z2(c, {no, nv}), Z3(c, {no, no}), Z4(c, {nv, nv});
    contract(c, "mnef,nf->me", 1.0, X2, l1, 0.0, Z1);
    contract(c, "me,imae->ia", 2.0, Z1, Lv, 1.0, R1);
    contract(c, "mnef,ne->mf", 1.0, X2, l1, 0.0, Z2);
    contract(c, "mf,imaf->ia", -1.0, Z2, Lv, 1.0, R1);
    contract(c, "mnef,mief->ni", 1.0, X2, Lv, 0.0, Z3);
    contract(c, "ni,na->ia", -1.0, Z3, l1, 1.0, R1);
    contract(c, "mnef,nmfa->ea", 1.0, X2, Lv, 0.0, Z4);
    contract(c, "ie,ea->ia", -1.0, l1, Z4, 1.0, R1);
  }
  {  // (s)
    Temp S(c, {no, no, no, nv});
    contract(c, "me,nief->mnif", 1.0, X1, l2, 0.0, S);
    contract(c, "mnif,mfna->ia", -1.0, S, Hovov, 1.0, R1);
    Temp S2(c, {no, nv, no, no});
    contract(c, "me,ifne->ifnm", 1.0, X1, Hovov, 0.0, S2);
    contract(c, "ifnm,nmaf->ia", -1.0, S2, l2, 1.0, R1);
    contract(c, "me,nife->mnif", 1.0, X1, l2, 0.0, S);
    contract(c, "mnif,mfan->ia", -1.0, S, Hovvo, 1.0, R1);
    contract(c, "me,ifen->ifnm", 1.0, X1, Hovvo, 0.0, S2);
    contract(c, "ifnm,nmfa->ia", -1.0, S2, l2, 1.0, R1);
    Temp S5(c, {no, nv, nv, nv});
    contract(c, "me,fgae->mfga", 1.0, X1, Hvvvv, 0.0, S5);
    contract(c, "mfga,imfg->ia", 0.5, S5, l2, 1.0, R1);
    contract(c, "me,fgea->mfga", 1.0, X1, Hvvvv, 0.0, S5);
    contract(c, "mfga,mifg->ia", 0.5, S5, l2, 1.0, R1);
    Temp S7(c, {no, no, no, nv});
    contract(c, "me,imno->inoe", 1.0, X1, Hoooo, 0.0, S7);
    contract(c, "inoe,noae->ia", 0.5, S7, l2, 1.0, R1);
    contract(c, "me,mino->inoe", 1.0, X1, Hoooo, 0.0, S7);
    contract(c, "inoe,noea->ia", 0.5, S7, l2, 1.0, R1);
  }
  {  // three-body terms, ccpert.cc:689-699 (O(no^4 nv^4) as written)
    Temp Gfb(c, {nv, nv}), Gfa(c, {nv, nv}), Gni(c, {no, no}), Gnj(c, {no, no});
    contract(c, "jmfe,jmbe->fb", 1.0, t2, l2, 0.0, Gfb);
    contract(c, "jnfb,jnab->fa", 1.0, t2, l2, 0.0, Gfa);
    contract(c, "jnfb,jifb->ni", 1.0, t2, l2, 0.0, Gni);
    contract(c, "nmeb,jmeb->nj", 1.0, t2, l2, 0.0, Gnj);
    Temp K1(c, {no, nv}), K2(c, {no, nv}), K3(c, {no, nv}), K4(c, {no, nv});
    contract(c, "nb,fb->nf", 1.0, X1, Gfb, 0.0, K1);
    contract(c, "inaf,nf->ia", -1.0, Lv, K1, 1.0, R1);
    contract(c, "mief,me->if", 1.0, Lv, X1, 0.0, K2);
    contract(c, "if,fa->ia", -1.0, K2, Gfa, 1.0, R1);
    contract(c, "mnea,me->na", 1.0, Lv, X1, 0.0, K3);
    contract(c, "ni,na->ia", -1.0, Gni, K3, 1.0, R1);
    contract(c, "nj,jf->nf", 1.0, Gnj, X1, 0.0, K4);
    contract(c, "inaf,nf->ia", -1.0, Lv, K4, 1.0, R1);
  }
  {  // (t)
    Temp V1(c, {no, no}), V2(c, {nv, nv});
    contract(c, "mnef,nife->mi", 1.0, X2, l2, 0.0, V1);
    contract(c, "mi,ma->ia", -1.0, V1, Hov, 1.0, R1);
    contract(c, "mnef,nmfa->ea", 1.0, X2, l2, 0.0, V2);
    contract(c, "ie,ea->ia", -1.0, Hov, V2, 1.0, R1);
    Temp Pn(c, {no, nv, no, nv});
    contract(c, "mnef,imfg->neig", 1.0, X2, l2, 0.0, Pn);
    contract(c, "neig,gnea->ia", -1.0, Pn, Hvovv, 1.0, R1);
    contract(c, "mnef,mifg->neig", 1.0, X2, l2, 0.0, Pn);
    contract(c, "neig,gnae->ia", -1.0, Pn, Hvovv, 1.0, R1);
    Temp Qm(c, {no, no, nv, no});
    contract(c, "mnef,gief->mngi", 1.0, X2, Hvovv, 0.0, Qm);
    contract(c, "mngi,nmag->ia", -1.0, Qm, l2, 1.0, R1);
    contract(c, "mnef,nifg->meig", 1.0, X2, l2, 0.0, Pn);
    contract(c, "meig,gmae->ia", 1.0, Pn, Hvovv_x, 1.0, R1);
    Temp P5(c, {nv, nv});
    contract(c, "mnef,nmfg->eg", 1.0, X2, l2, 0.0, P5);
    contract(c, "eg,giea->ia", 1.0, P5, Hvovv_x, 1.0, R1);
    Temp P6(c, {no, no, no, no});
    contract(c, "mnef,oief->mnoi", 1.0, X2, l2, 0.0, P6);
    contract(c, "mnoi,mnoa->ia", 1.0, P6, Hooov, 1.0, R1);
    Temp P7(c, {no, nv, no, nv});
    contract(c, "mnef,omaf->neoa", 1.0, X2, l2, 0.0, P7);
    contract(c, "neoa,inoe->ia", 1.0, P7, Hooov, 1.0, R1);
    contract(c, "mnef,onea->mfoa", 1.0, X2, l2, 0.0, P7);
    contract(c, "mfoa,miof->ia", 1.0, P7, Hooov, 1.0, R1);
    Temp P9(c, {no, no});
    contract(c, "mnef,nofe->mo", 1.0, X2, l2, 0.0, P9);
    contract(c, "mo,mioa->ia", -1.0, P9, Hooov_x, 1.0, R1);
    contract(c, "mnef,nofa->meoa", 1.0, X2, l2, 0.0, P7);
    contract(c, "meoa,imoe->ia", -1.0, P7, Hooov_x, 1.0, R1);
  }

  // ---------------- Y2 ----------------
  Temp Q(c, {no, no, nv, nv});
  axpby(c, Q->size(), 0.5 * w, Y2o.p, 0.0, Q->p);
  contract(c, "ia,jb->ijab", 2.0, Y1o, Hov, 1.0, Q);
  contract(c, "ja,ib->ijab", -1.0, Y1o, Hov, 1.0, Q);
  contract(c, "ijeb,ea->ijab", 1.0, Y2o, Hvv, 1.0, Q);
  contract(c, "mjab,im->ijab", -1.0, Y2o, Hoo, 1.0, Q);
  contract(c, "mnab,ijmn->ijab", 0.5, Y2o, Hoooo, 1.0, Q);
  // 0.5 sum_ef Y2_ijef Hvvvv_efab, moved past the symmetrisation: W_abef = Hvvvv_efab + Hvvvv_feba
  const bool packed = hbar_ladder_packed(c);
  if (!packed) contract(c, "ijef,efab->ijab", 0.5, Y2o, Hvvvv, 1.0, Q);
  contract(c, "ie,ejab->ijab", 1.0, Y1o, Hvovv_x, 1.0, Q);
  contract(c, "mb,jima->ijab", -1.0, Y1o, Hooov_x, 1.0, Q);
  contract(c, "mjeb,ieam->ijab", 1.0, Y2o, Hovvo_x, 1.0, Q);
  contract(c, "mibe,jema->ijab", -1.0, Y2o, Hovov, 1.0, Q);
  contract(c, "mieb,jeam->ijab", -1.0, Y2o, Hovvo, 1.0, Q);
  contract(c, "ae,ijeb->ijab", 1.0, Gvv, Lv, 1.0, Q);
  contract(c, "mi,mjab->ijab", -1.0, Goo, Lv, 1.0, Q);
  contract(c, "jb,ia->ijab", 2.0, l1, pov, 1.0, Q);                       // (o)
  contract(c, "ib,ja->ijab", -1.0, l1, pov, 1.0, Q);
  contract(c, "ijeb,ea->ijab", 1.0, l2, Avv, 1.0, Q);                     // (p)
  contract(c, "mjab,im->ijab", -1.0, l2, Aoo, 1.0, Q);
  {  // (u)
    Temp U1(c, {no, nv}), U2(c, {nv, nv}), U3(c, {no, no}), U4(c, {no, nv});
    contract(c, "me,mieb->ib", 1.0, X1, Lv, 0.0, U1);
    contract(c, "ja,ib->ijab", -1.0, l1, U1, 1.0, Q);
    contract(c, "me,mb->eb", 1.0, X1, l1, 0.0, U2);
    contract(c, "ijae,eb->ijab", -1.0, Lv, U2, 1.0, Q);
    contract(c, "me,ie->mi", 1.0, X1, l1, 0.0, U3);
    contract(c, "mi,jmba->ijab", -1.0, U3, Lv, 1.0, Q);
    contract(c, "me,imae->ia", 1.0, X1, Lv, 0.0, U4);
    contract(c, "ia,jb->ijab", 2.0, U4, l1, 1.0, Q);
  }
  {  // (w)
    Temp W1(c, {nv, nv}), W2(c, {no, no});
    contract(c, "ma,me->ae", 1.0, Hov, X1, 0.0, W1);
    contract(c, "jibe,ae->ijab", -1.0, l2, W1, 1.0, Q);
    contract(c, "ie,me->im", 1.0, Hov, X1, 0.0, W2);
    contract(c, "im,jmba->ijab", -1.0, W2, l2, 1.0, Q);
    Temp Qa(c, {no, no, no, nv});
    contract(c, "me,jife->mjif", 1.0, X1, l2, 0.0, Qa);
    contract(c, "mjif,fmba->ijab", -1.0, Qa, Hvovv, 1.0, Q);
    Temp Qb(c, {nv, no, nv, no});
    contract(c, "fjea,me->fjam", 1.0, Hvovv, X1, 0.0, Qb);
    contract(c, "fjam,mifb->ijab", -1.0, Qb, l2, 1.0, Q);
    contract(c, "fibe,me->fibm", 1.0, Hvovv, X1, 0.0, Qb);
    contract(c, "fibm,jmfa->ijab", -1.0, Qb, l2, 1.0, Q);
    Temp Q4(c, {nv, nv});
    contract(c, "fmae,me->fa", 1.0, Hvovv_x, X1, 0.0, Q4);
    contract(c, "fa,jibf->ijab", 1.0, Q4, l2, 1.0, Q);
    contract(c, "fiea,me->fiam", 1.0, Hvovv_x, X1, 0.0, Qb);
    contract(c, "fiam,jmbf->ijab", 1.0, Qb, l2, 1.0, Q);
    Temp Qc(c, {no, no, nv, no});
    contract(c, "nibe,me->nibm", 1.0, l2, X1, 0.0, Qc);
    contract(c, "jmna,nibm->ijab", 1.0, Hooov, Qc, 1.0, Q);
    contract(c, "nieb,me->nibm", 1.0, l2, X1, 0.0, Qc);
    contract(c, "mjna,nibm->ijab", 1.0, Hooov, Qc, 1.0, Q);
    Temp Q8(c, {no, no, no, no});
    contract(c, "jine,me->jinm", 1.0, Hooov, X1, 0.0, Q8);
    contract(c, "jinm,nmba->ijab", 1.0, Q8, l2, 1.0, Q);
    contract(c, "jnbe,me->jnbm", 1.0, l2, X1, 0.0, Qc);
    contract(c, "mina,jnbm->ijab", -1.0, Hooov_x, Qc, 1.0, Q);
    Temp Q10(c, {no, no});
    contract(c, "imne,me->in", 1.0, Hooov_x, X1, 0.0, Q10);
    contract(c, "in,jnba->ijab", -1.0, Q10, l2, 1.0, Q);
  }
  {  // (x), ccpert.cc:834-872 (O(no^4 nv^4) as written)
    Temp Zo(c, {no, no, no, no});
    contract(c, "jief,mnef->jimn", 1.0, l2, X2, 0.0, Zo);
    contract(c, "nmab,jimn->ijab", 0.25, Vv, Zo, 1.0, Q);
    contract(c, "jife,mnef->jimn", 1.0, l2, X2, 0.0, Zo);
    contract(c, "mnab,jimn->ijab", 0.25, Vv, Zo, 1.0, Q);
    Temp Zm(c, {no, nv, no, nv});
    contract(c, "mifb,mnef->ibne", 1.0, l2, X2, 0.0, Zm);
    contract(c, "jnae,ibne->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "nieb,mnef->ibmf", 1.0, l2, X2, 0.0, Zm);
    contract(c, "jmaf,ibmf->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "mibf,mnef->ibne", 1.0, l2, X2, 0.0, Zm);
    contract(c, "njae,ibne->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "nibe,mnef->ibmf", 1.0, l2, X2, 0.0, Zm);
    contract(c, "mjaf,ibmf->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "imfb,mnef->ibne", 1.0, l2, X2, 0.0, Zm);
    contract(c, "jnea,ibne->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "ineb,mnef->ibmf", 1.0, l2, X2, 0.0, Zm);
    contract(c, "jmfa,ibmf->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "imbf,mnef->ibne", 1.0, l2, X2, 0.0, Zm);
    contract(c, "njea,ibne->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "inbe,mnef->ibmf", 1.0, l2, X2, 0.0, Zm);
    contract(c, "mjfa,ibmf->ijab", 0.25, Vv, Zm, 1.0, Q);
    contract(c, "jief,mnef->jimn", 1.0, Vv, X2, 0.0, Zo);
    contract(c, "jimn,nmab->ijab", 0.25, Zo, l2, 1.0, Q);
    contract(c, "jife,mnef->jimn", 1.0, Vv, X2, 0.0, Zo);
    contract(c, "jimn,mnab->ijab", 0.25, Zo, l2, 1.0, Q);
    contract(c, "jnbe,mnef->jbmf", 1.0, l2, X2, 0.0, Zm);
    contract(c, "imaf,jbmf->ijab", -0.5, Lv, Zm, 1.0, Q);
    contract(c, "jmbf,mnef->jbne", 1.0, l2, X2, 0.0, Zm);
    contract(c, "inae,jbne->ijab", -0.5, Lv, Zm, 1.0, Q);
    Temp Zin(c, {no, no}), Zaf(c, {nv, nv});
    contract(c, "mief,mnef->in", 1.0, Lv, X2, 0.0, Zin);
    contract(c, "in,jnba->ijab", -0.5, Zin, l2, 1.0, Q);
    contract(c, "mnea,mnef->af", 1.0, Lv, X2, 0.0, Zaf);
    contract(c, "af,jibf->ijab", -0.5, Zaf, l2, 1.0, Q);
    contract(c, "nmfa,mnef->ae", 1.0, Lv, X2, 0.0, Zaf);
    contract(c, "ae,jibe->ijab", -0.5, Zaf, l2, 1.0, Q);
    contract(c, "nife,mnef->im", 1.0, Lv, X2, 0.0, Zin);
    contract(c, "im,jmba->ijab", -0.5, Zin, l2, 1.0, Q);
    contract(c, "nmfb,mnef->eb", 1.0, l2, X2, 0.0, Zaf);
    contract(c, "ijae,eb->ijab", -1.0, Lv, Zaf, 1.0, Q);
    contract(c, "njfe,mnef->jm", 1.0, l2, X2, 0.0, Zin);
    contract(c, "imab,jm->ijab", -1.0, Lv, Zin, 1.0, Q);
    contract(c, "nifb,mnef->ibme", 1.0, l2, X2, 0.0, Zm);
    contract(c, "mjea,ibme->ijab", -1.0, Lv, Zm, 1.0, Q);
    contract(c, "njfb,mnef->jbme", 1.0, l2, X2, 0.0, Zm);
    contract(c, "imae,jbme->ijab", 2.0, Lv, Zm, 1.0, Q);
  }
  copy_into(c, Q, R2);
  transpose_add(c, "jiba->ijab", 1.0, Q, 1.0, R2);
  if (packed) packed_ladder(c, 0.5, Y2o, "Hvvvv", 1, "Hpp1", "Hmm1", R2.p);
}

double pseudoresponse(Ctx& c, Perturbation& p, double* amps) {  // ccpert.cc:233-253
  const int no = c.no, nv = c.nv;
  Tensor X1 = amp1(c, amps), X2 = amp2(c, amps);
  double p1 = 2.0 * dot_all(c, X1, view(P(c, p, "Avo"), "ai->ia"));
  Temp X(c, {no, no, nv, nv});
  transpose_add(c, "ijab->ijba", -1.0, X2, 0.0, X);
  axpby(c, X->size(), 2.0, X2.p, 1.0, X->p);
  double p2 = 2.0 * dot_all(c, X, view(P(c, p, "Avvoo"), "abij->ijab"));
  return -2.0 * (p1 + p2);
}
}  // namespace

int pert_create(Ctx& c, const double* pert, double omega) {
  UCC_REQUIRE(c.have_lambda, UCC_BAD_STATE, "perturbed wavefunctions need HBAR and Lambda");
  Fp64Scope fp64(c);
  const int no = c.no, nv = c.nv, n = no + nv;
  auto pp = std::make_unique<Perturbation>();
  pp->id = (int)c.perts.size();
  pp->omega = omega;
  pp->pfx = "P" + std::to_string(pp->id) + ":";
  Perturbation& p = *pp;
  auto put = [&](const char* nm, int r0, int nr, int c0, int nc) {
    std::vector<double> h((size_t)nr * nc);
    for (int i = 0; i < nr; i++)
      for (int j = 0; j < nc; j++) h[(size_t)i * nc + j] = pert[(size_t)(r0 + i) * n + c0 + j];
    Tensor t = c.alloc(p.pfx + nm, {nr, nc}, false);
    UCC_CUDA(cudaMemcpyAsync(t.p, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
  };
  put("poo", 0, no, 0, no);
  put("pov", 0, no, no, nv);
  put("pvo", no, nv, 0, no);
  put("pvv", no, nv, no, nv);
  pertbar(c, p);
  // guesses X = Y = A / (D + omega) with D from the HBAR diagonals, ccpert.cc:57-73
  const int64_t np = npacked(c);
  Tensor X = c.alloc(p.pfx + "X", {np}, false);
  c.alloc(p.pfx + "Xold", {np}, false);
  Tensor Y = c.alloc(p.pfx + "Y", {np}, false);
  c.alloc(p.pfx + "Yold", {np}, false);
  {
    Temp R0(c, {np}, true), Z(c, {np}, true);
    transpose_add(c, "ai->ia", 1.0, P(c, p, "Avo"), 0.0, amp1(c, R0->p));
    Tensor R2 = amp2(c, R0->p);
    transpose_add(c, "abij->ijab", 1.0, P(c, p, "Avvoo"), 0.0, R2);
    transpose_add(c, "baji->ijab", 1.0, P(c, p, "Avvoo"), 1.0, R2);
    Tensor hd = c.get("Hdiag");
    Scratch ss(c, sizeof(double));
    jacobi_update(c, no, nv, hd.p, hd.p + no, omega, R0->p, R0->p + (int64_t)no * nv, Z->p, Z->p + (int64_t)no * nv,
                  X.p, X.p + (int64_t)no * nv, ss.d());
    UCC_CUDA(cudaMemcpyAsync(Y.p, X.p, sizeof(double) * np, cudaMemcpyDeviceToDevice, c.stream));
  }
  UCC_CUDA(cudaStreamSynchronize(c.stream));
  c.perts.push_back(std::move(pp));
  return (int)c.perts.size() - 1;
}

CCSDResult pert_solve(Ctx& c, int h, bool right) {  // ccpert.cc:177-229
  Perturbation& p = get_pert(c, h);
  Fp64Scope fp64(c);
  UCC_REQUIRE(right || p.right_done, UCC_BAD_STATE, "left-hand solve needs the right-hand solution");
  const int no = c.no, nv = c.nv;
  const int64_t np = npacked(c), n1 = (int64_t)no * nv;
  const std::string cur = p.pfx + (right ? "X" : "Y"), old = p.pfx + (right ? "Xold" : "Yold");
  Tensor hd = c.get("Hdiag");
  Scratch sumsq(c, sizeof(double));
  Temp R(c, {np});
  Diis diis(c, np, 8);
  if (c.opt.print) {
    std::printf("\n\tCoupled-Cluster %s Perturbed Wfn Iteration:\n", right ? "RH" : "LH");
    std::printf("\t-------------------------------------\n\t Iter   Pseudoresponse      RMS   \n");
    std::printf("\t-------------------------------------\n\t  %3d  %20.15f\n", 0, pseudoresponse(c, p, c.get(cur).p));
  }
  double rms = INFINITY;
  bool converged = false;
  MixedSweeps sw(c);  // MIXED: split, record and delta sweeps; X2/Y2 are symmetrised by construction
  int iter;
  for (iter = 1; iter <= c.opt.maxiter; iter++) {
    c.store[cur].swap(c.store[old]);
    double* o = c.get(old).p;
    double* nw = c.get(cur).p;
    const MixedSweeps::Kind kind = sw.begin();
    {
      PrecisionScope scope(c, kind != MixedSweeps::kSplit);
      if (right)
        build_X(c, p, amp1(c, o), amp2(c, o), amp1(c, R->p), amp2(c, R->p));
      else
        build_Y(c, p, amp1(c, o), amp2(c, o), amp1(c, R->p), amp2(c, R->p));
    }
    sw.end();
    jacobi_update(c, no, nv, hd.p, hd.p + no, p.omega, R->p, R->p + n1, o, o + n1, nw, nw + n1, sumsq.d());
    double ss = 0.0;
    UCC_CUDA(cudaMemcpyAsync(&ss, sumsq.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream));
    UCC_CUDA(cudaStreamSynchronize(c.stream));
    rms = std::sqrt(ss);
    tc_check(c);
    UCC_REQUIRE(std::isfinite(rms), UCC_NAN_DETECTED, "perturbed-wavefunction residual is not finite");
    bool restart = false;
    if (sw.after(rms, &restart)) {
      converged = true;
      break;
    }
    if (restart) diis.reset();
    if (c.opt.diis && !restart) {
      diis.add(nw, o);
      if (diis.size() > 2) diis.extrapolate(nw);
    }
    if (c.opt.print) {
      static const char* tag[] = {"", " split", " record", " delta"};
      std::printf("\t  %3d  %20.15f  %5.3e%s\n", iter, pseudoresponse(c, p, nw), rms, tag[kind]);
    }
  }
  CCSDResult res;
  res.iterations = std::min(iter, c.opt.maxiter);
  res.converged = converged;
  res.e_ccsd = pseudoresponse(c, p, c.get(cur).p);
  if (res.converged) (right ? p.right_done : p.left_done) = true;
  return res;
}

double linresp(Ctx& c, int hx, int hy) {  // ccresp.cc:28-124
  Perturbation& X = get_pert(c, hx);
  Fp64Scope fp64(c);
  Perturbation& Y = get_pert(c, hy);
  const int no = c.no, nv = c.nv;
  double* Lp = c.get("Lam").p;
  Tensor l1 = amp1(c, Lp), l2 = amp2(c, Lp);
  double* yx = c.get(Y.pfx + "X").p;
  double* yy = c.get(Y.pfx + "Y").p;
  Tensor X1y = amp1(c, yx), X2y = amp2(c, yx), Y1y = amp1(c, yy), Y2y = amp2(c, yy);
  Tensor Avo = P(c, X, "Avo"), Avv = P(c, X, "Avv"), Aoo = P(c, X, "Aoo"), Avvoo = P(c, X, "Avvoo");
  Tensor Avvvo = P(c, X, "Avvvo"), Aovoo = P(c, X, "Aovoo"), pov = P(c, X, "pov");
  double polar1 = dot_all(c, view(Avo, "ai->ia"), Y1y);
  {
    Temp Ax(c, {no, no, nv, nv});
    transpose_add(c, "abij->ijab", 1.0, Avvoo, 0.0, Ax);
    transpose_add(c, "baji->ijab", 1.0, Avvoo, 1.0, Ax);
    polar1 += 0.5 * dot_all(c, Ax, Y2y);
  }
  double polar2 = 0.0;
  {
    Temp X(c, {no, no, nv, nv}), M(c, {no, nv});
    transpose_add(c, "ijab->ijba", -1.0, X2y, 0.0, X);
    axpby(c, X->size(), 2.0, X2y.p, 1.0, X->p);
    contract(c, "jb,ijab->ia", 1.0, pov, X, 0.0, M);
    polar2 += dot_all(c, l1, M);
    contract(c, "ac,ic->ia", 1.0, Avv, X1y, 0.0, M);
    polar2 += dot_all(c, l1, M);
    contract(c, "ki,ka->ia", 1.0, Aoo, X1y, 0.0, M);
    polar2 -= dot_all(c, l1, M);
    Temp A(c, {no, nv});  // A[i,a] = l2[i,j,b,c] Avvvo[b,c,a,j]
    contract(c, "ijbc,bcaj->ia", 1.0, l2, Avvvo, 0.0, A);
    polar2 += dot_all(c, A, X1y);
    Temp B(c, {no, nv});  // B[k,a] = l2[i,j,a,b] Aovoo[k,b,i,j]
    contract(c, "ijab,kbij->ka", 1.0, l2, Aovoo, 0.0, B);
    polar2 -= 0.5 * dot_all(c, B, X1y);
    contract(c, "ijab,kaji->kb", 1.0, l2, Aovoo, 0.0, B);
    polar2 -= 0.5 * dot_all(c, B, X1y);
    Temp G(c, {no, no});  // G[k,i] = l2[i,j,a,b] X2y[k,j,a,b]
    contract(c, "ijab,kjab->ki", 1.0, l2, X2y, 0.0, G);
    polar2 -= 0.5 * dot_all(c, G, Aoo);
    contract(c, "ijab,kiba->kj", 1.0, l2, X2y, 0.0, G);
    polar2 -= 0.5 * dot_all(c, G, Aoo);
    Temp H(c, {nv, nv});  // H[b,c] = l2[i,j,a,b] X2y[i,j,a,c]
    contract(c, "ijab,ijac->bc", 1.0, l2, X2y, 0.0, H);
    polar2 += 0.5 * dot_all(c, H, Avv);
    contract(c, "ijab,jibc->ac", 1.0, l2, X2y, 0.0, H);
    polar2 += 0.5 * dot_all(c, H, Avv);
    polar2 += 2.0 * dot_all(c, pov, X1y);
  }
  return -(polar1 + polar2);
}

// ---------------------------------------------------------------------------------------
// named tensors for ucc_get_tensor / ucc_set_tensor
// ---------------------------------------------------------------------------------------
Tensor named_tensor(Ctx& c, const std::string& name) {
  auto colon = name.find(':');
  if (colon != std::string::npos) {
    const std::string what = name.substr(0, colon);
    const int h = std::atoi(name.c_str() + colon + 1);
    Perturbation& p = get_pert(c, h);
    if (what == "X1") return amp1(c, c.get(p.pfx + "X").p);
    if (what == "X2") return amp2(c, c.get(p.pfx + "X").p);
    if (what == "Y1") return amp1(c, c.get(p.pfx + "Y").p);
    if (what == "Y2") return amp2(c, c.get(p.pfx + "Y").p);
    throw Error(UCC_BAD_ARGS, "unknown tensor " + name);
  }
  if (name == "t2_guess") return amp2(c, c.get("T_guess").p);  // the pending guess of the next CCSD solve
  if (name == "t1") return amp1(c, c.get("T").p);
  if (name == "t2") return amp2(c, c.get("T").p);
  if (name == "l1") return amp1(c, c.get("Lam").p);
  if (name == "l2") return amp2(c, c.get("Lam").p);
  if (name == "s1") return c.get("TS1");
  if (name == "s2") return c.get("TS2");
  static const char* tg[][2] = {{"DooT", "TDoo"},     {"DvvT", "TDvv"},     {"DovT", "TDov"},
                                {"GoovvT", "TGoovv"}, {"GooovT", "TGooov"}, {"GvvvoT", "TGvvvo"}};
  for (auto& p : tg)
    if (name == p[0]) return c.get(p[1]);
  static const char* direct[] = {"tau",   "Doo",   "Dvv",   "Dov",   "Dvo",   "Hov",   "Hoo",   "Hvv",
                                 "Hoooo", "Hvvvv", "Hvovv", "Hooov", "Hovvo", "Hovov", "Hvvvo", "Hovoo",
                                 "Goooo", "Gvvvv", "Gooov", "Gvvvo", "Govov", "Goovv"};
  for (const char* d : direct)
    if (name == d) return c.get(name);
  throw Error(UCC_BAD_ARGS, "unknown tensor " + name);
}

void set_named_tensor(Ctx& c, const std::string& name, const double* host, size_t count) {
  const int no = c.no, nv = c.nv;
  const int64_t n1 = (int64_t)no * nv, n2 = (int64_t)no * no * nv * nv;
  const bool lam = name == "l1" || name == "l2";
  UCC_REQUIRE(name == "t1" || name == "t2" || lam, UCC_BAD_ARGS, "settable tensors: t1 t2 l1 l2");
  const int64_t want = (name == "t1" || name == "l1") ? n1 : n2;
  UCC_REQUIRE((int64_t)count == want, UCC_BAD_ARGS, "size mismatch for " + name);
  const std::string g = lam ? "Lam_guess" : "T_guess";
  if (!c.has(g)) c.alloc(g, {n1 + n2}, true);
  double* dst = c.get(g).p + ((name == "t1" || name == "l1") ? 0 : n1);
  UCC_CUDA(cudaMemcpyAsync(dst, host, sizeof(double) * count, cudaMemcpyHostToDevice, c.stream));
  UCC_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace ucc
