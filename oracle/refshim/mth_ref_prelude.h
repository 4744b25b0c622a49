/*
 * Forced first include when compiling the reference sources here.  Defining
 * the include guard of src/evpFlags.h makes the compiler skip that file, so
 * the physics flags below are the build's configuration: the shipped set
 * (src/evpFlags.h:4-40) minus DD_CU, whose hard-coded Cu constants
 * (src/init.c:821-825) would override the elastic constants of input.in.
 */
#ifndef MTH_REF_PRELUDE_H
#define MTH_REF_PRELUDE_H
#define EVPFLAGS_H
#define NPHMAX 2
#define NSYSMX 12
#define DD_BASED_FLAG
#define FORWARD_PLUS_BACKWARD
#define NR_MODIFIED
#define DD_GND
#define DD_GND_FIRST_ORDER
#define PF_DRX
#define GB_BULGING_ONLY

/*
 * With MTH_PF_HOOK (only for the copy of src/pf_xrx.c linked into
 * oracle/_ref/drx_ref): the phase-field grid type is a subclass of the
 * reference's PFgrid3D (src/PFgrid.h:123-130) whose swap() -- called once
 * per substep, at the end of Update_grid (src/pf_xrx.c:1296) -- hands the
 * freshly updated grid to mth_ref_pf_after_substep, which records every
 * voxel's (id, eta) list in its stored order.  Nothing else of the grid
 * changes: storage, operator[] and the insertion rule are the reference's.
 */
#ifdef MTH_PF_HOOK
#include "PFgrid.h"
typedef PFgrid3D MthPFgrid3DBase;
void mth_ref_pf_after_substep(MthPFgrid3DBase& g, int l_x, int l_y, int l_z);
class MthPFgrid3D : public MthPFgrid3DBase {
 public:
  MthPFgrid3D(int x, int y, int z) : MthPFgrid3DBase(x, y, z), lx_(x), ly_(y), lz_(z) {}
  void swap(MthPFgrid3D& g) {
    MthPFgrid3DBase::swap(g);
    mth_ref_pf_after_substep(*this, lx_, ly_, lz_);
  }

 private:
  int lx_, ly_, lz_;
};
#define PFgrid3D MthPFgrid3D
#endif
#endif
