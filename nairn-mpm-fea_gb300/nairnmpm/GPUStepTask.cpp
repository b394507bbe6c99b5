/*
 * GPUStepTask.cpp -- see GPUStepTask.hpp.
 */
#include "stdafx.h"

#include <cmath>
#include <cstring>
#include <string>

#include "nairnmpm/GPUStepTask.hpp"
#include "NairnMPM_Class/NairnMPM.hpp"
#include "NairnMPM_Class/MeshInfo.hpp"
#include "MPM_Classes/MPMBase.hpp"
#include "Materials/MaterialBase.hpp"
#include "Materials/ContactLaw.hpp"
#include "Elements/ElementBase.hpp"
#include "Nodes/NodalPoint.hpp"
#include "Boundary_Conditions/NodalVelBC.hpp"
#include "System/ArchiveData.hpp"
#include "Custom_Tasks/CustomTask.hpp"
#include "Exceptions/CommonException.hpp"

namespace {

// The input value x whose conversion x * scale -- the product the XML reader
// and the ABI both form -- gives back the stored value exactly (stored /
// scale itself may be an ulp off), so the device derives its constants from
// the same doubles as the reference.
double Unscale(double stored, double scale)
{	double x = stored / scale;
	for(int k = 0; k < 4 && x * scale != stored; k++)
		x = nextafter(x, x * scale < stored ? (scale > 0. ? HUGE_VAL : -HUGE_VAL) : (scale > 0. ? -HUGE_VAL : HUGE_VAL));
	return x;
}

// An input property of a material by its XML name, through the same public
// accessor the XML reader fills it with (MaterialBase::InputMaterialProperty):
// the value in the units the XML gives it (MPa for moduli and stresses).
double InputProperty(MaterialBase *m, const char *name)
{	char key[64];
	strncpy(key, name, sizeof(key) - 1);
	key[sizeof(key) - 1] = 0;
	int input = 0;
	double scale = 1.;
	char *ptr = m->InputMaterialProperty(key, input, scale);
	if(ptr == NULL)
		throw CommonException((std::string("material property ") + name + " is not available for material type " +
		                       std::to_string(m->MaterialID())).c_str(), "GPUStepTask");
	if(input == INT_NUM) return (double)(*(int *)ptr);
	return Unscale(*(double *)ptr, scale != 0. ? scale : 1.);
}

}  // namespace

GPUStepTask::GPUStepTask(const char *name) : MPMTask(name)
{
	ctx = NULL;
	hostStale = false;
	dim = fmobj->IsThreeD() ? 3 : 2;

	// grid (MeshInfo and the node coordinates of nd[], nodes numbered x fastest)
	int nxn = 0, nyn = 0, nzn = 0;
	mpmgrid.GetGridPoints(&nxn, &nyn, &nzn);
	MpmGpuGrid g;
	memset(&g, 0, sizeof(g));
	g.dim = dim;
	g.nx = nxn - 1;
	g.ny = nyn - 1;
	g.nz = dim == 3 ? nzn - 1 : 0;
	Vector cell = mpmgrid.GetCellSize();
	g.xmin = mpmgrid.xmin;
	g.ymin = mpmgrid.ymin;
	g.zmin = dim == 3 ? mpmgrid.zmin : 0.;
	g.dx = cell.x;
	g.dy = cell.y;
	g.dz = dim == 3 ? cell.z : 0.;
	g.thickness = dim == 3 ? 1. : mpmgrid.GetThickness();
	std::vector<double> xn(nxn), yn(nyn), zn(dim == 3 ? nzn : 0);
	for(int i = 0; i < nxn; i++) xn[i] = nd[1 + i]->x;
	for(int j = 0; j < nyn; j++) yn[j] = nd[1 + j * nxn]->y;
	for(int k = 0; k < (int)zn.size(); k++) zn[k] = nd[1 + k * nxn * nyn]->z;
	g.xnodes = xn.data();
	g.ynodes = yn.data();
	g.znodes = dim == 3 ? zn.data() : NULL;

	// analysis options
	if(theTasks != NULL)
		throw CommonException("custom tasks are not passed to the GPU step by this binding", "GPUStepTask");
	MpmGpuOptions o;
	memset(&o, 0, sizeof(o));
	o.np = fmobj->np;                            // PLANE_STRAIN_MPM or THREED_MPM
	o.method = fmobj->mpmApproach;               // USF, USAVG or USL
	o.shape = ElementBase::useGimp;              // the GIMP constants of the ABI
	o.precision = getenv("NAIRN_GPU_MIXED") ? MPMGPU_PREC_MIXED : MPMGPU_PREC_FP64;
	o.p2g = MPMGPU_P2G_ATOMIC;
	o.inc_defgrad_terms = MaterialBase::incrementalDefGradTerms;
	o.nfields = fmobj->multiMaterialMode ? maxMaterialFields : 1;
	o.sort_interval = 1;
	o.timestep = timestep;
	o.fraction_usf = fractionUSF;
	Check(mpmgpu_create(&g, &o, &ctx), "mpmgpu_create");

	// materials: type, field and input properties of each MaterialBase that
	// particles can use (contact laws are materials too, but hold no particles)
	std::vector<MpmGpuMaterial> mats;
	historyCount.assign(nmat, 0);
	deviceMat.assign(nmat, -1);
	for(int i = 0; i < nmat; i++)
	{	MaterialBase *m = theMaterials[i];
		if(m->MaterialStyle() == CONTACT_MAT) continue;
		deviceMat[i] = (int)mats.size();
		mats.emplace_back();
		MpmGpuMaterial &d = mats.back();
		memset(&d, 0, sizeof(d));
		d.type = m->MaterialID();
		d.field = fmobj->multiMaterialMode ? m->GetField() : 0;
		if(d.field < 0) d.field = 0;
		if(d.type == MPMGPU_MAT_RIGID_CONTACT) continue;
		d.rho = Unscale(m->GetRho(NULL), 0.001);   // g/mm^3 -> g/cm^3
		if(d.type == MPMGPU_MAT_NEOHOOKEAN)
		{	d.G = InputProperty(m, "G");
			d.K = InputProperty(m, "K");
			d.UJOption = (int32_t)InputProperty(m, "UJOption");
			historyCount[i] = 2;                  // J, Jres
		}
		else
		{	d.E = InputProperty(m, "E");
			d.nu = InputProperty(m, "nu");
			if(d.type == MPMGPU_MAT_ISOPLASTICITY)
			{	d.yield = InputProperty(m, "yield");
				d.Ep = InputProperty(m, "Ep");
				historyCount[i] = 1;              // cumulative plastic strain
			}
		}
	}
	Check(mpmgpu_set_materials(ctx, mats.data(), (int32_t)mats.size()), "mpmgpu_set_materials");

	// multimaterial mode: the normal method and the Coulomb law's coefficient
	if(fmobj->multiMaterialMode)
	{	MpmGpuContact c;
		memset(&c, 0, sizeof(c));
		c.enabled = 1;
		c.normals = mpmgrid.materialNormalMethod;
		ContactLaw *law = mpmgrid.GetMaterialContactLaw(0, 1);
		int input = 0;
		double scale = 1.;
		char key[] = "coeff";
		char *ptr = law != NULL ? law->InputContactProperty(key, input, scale) : NULL;
		if(ptr == NULL) throw CommonException("only Coulomb friction contact is bound", "GPUStepTask");
		c.friction = *(double *)ptr;
		c.contact_cutoff = mpmgrid.contactByDisplacements ? -1. : mpmgrid.positionCutoff;
		c.rigid_gradient_bias = sqrt(mpmgrid.rigidGradientBias);  // MeshInfo holds it squared
		Check(mpmgpu_set_contact(ctx, &c), "mpmgpu_set_contact");
	}

	// velocity conditions in firstVelocityBC list order
	std::vector<MpmGpuVelBC> bcs;
	for(NodalVelBC *bc = firstVelocityBC; bc != NULL; bc = (NodalVelBC *)bc->GetNextObject())
	{	MpmGpuVelBC b;
		b.node = bc->GetNodeNum();
		b.dir = bc->GetSetDirection();
		b.value = bc->GetBCValue();
		b.ftime = bc->GetBCFirstTime();
		bcs.push_back(b);
	}
	Check(mpmgpu_set_velocity_bcs(ctx, bcs.empty() ? NULL : bcs.data(), (int32_t)bcs.size()),
	      "mpmgpu_set_velocity_bcs");

	PackParticles();
	Check(mpmgpu_upload_particles(ctx, &soa), "mpmgpu_upload_particles");
}

GPUStepTask::~GPUStepTask()
{	if(ctx != NULL) mpmgpu_destroy(ctx);
}

// a non-zero status becomes the reference's CommonException
void GPUStepTask::Check(int status, const char *where) const
{	if(status == MPMGPU_OK) return;
	throw CommonException(mpmgpu_last_error(ctx), where);
}

// one NairnMPM::MPMStep on the device
bool GPUStepTask::Execute(int taskOption)
{	Check(mpmgpu_step(ctx, 1, mtime), "mpmgpu_step");
	hostStale = true;
	// NairnMPM::CMAnalysis archives after the step when this is true
	// (ArchiveData::WillArchive, or the last step past maxtime)
	if(archiver->WillArchive() || mtime + timestep > fmobj->maxtime) SyncToHost();
	return true;
}

void GPUStepTask::SyncToHost(void)
{	if(!hostStale) return;
	Check(mpmgpu_download_particles(ctx, &soa), "mpmgpu_download_particles");
	UnpackParticles();
	hostStale = false;
}

// the column order of MpmGpuParticles (every double column, one block)
enum { C_X, C_Y, C_Z, C_VX, C_VY, C_VZ, C_X0, C_Y0, C_Z0, C_MASS, C_LPX, C_LPY, C_LPZ,
       C_EXX, C_EYY, C_EZZ, C_EXY, C_EXZ, C_EYZ, C_WXY, C_WXZ, C_WYZ,
       C_SXX, C_SYY, C_SZZ, C_SXY, C_SXZ, C_SYZ, C_P,
       C_PXX, C_PYY, C_PZZ, C_PXY, C_PXZ, C_PYZ, C_H0, C_H1, C_WORK, C_PLAST, C_COUNT };

void GPUStepTask::PackParticles(void)
{	const size_t n = (size_t)nmpms;
	cols.assign(n * C_COUNT, 0.);
	matCol.assign(n, 0);
	elemCol.assign(n, 0);
	double *c[C_COUNT];
	for(int k = 0; k < C_COUNT; k++) c[k] = cols.data() + k * n;
	for(size_t p = 0; p < n; p++)
	{	MPMBase *m = mpm[p];
		c[C_X][p] = m->pos.x; c[C_Y][p] = m->pos.y; c[C_Z][p] = m->pos.z;
		c[C_VX][p] = m->vel.x; c[C_VY][p] = m->vel.y; c[C_VZ][p] = m->vel.z;
		c[C_X0][p] = m->origpos.x; c[C_Y0][p] = m->origpos.y; c[C_Z0][p] = m->origpos.z;
		c[C_MASS][p] = m->mp;
		Vector lp;
		m->GetDimensionlessSize(lp);
		c[C_LPX][p] = lp.x; c[C_LPY][p] = lp.y; c[C_LPZ][p] = dim == 3 ? lp.z : 1.;
		Tensor *ep = m->GetStrainTensor(), *sp = m->GetStressTensor(), *pl = m->GetAltStrainTensor();
		TensorAntisym *w = m->GetRotationStrainTensor();
		c[C_EXX][p] = ep->xx; c[C_EYY][p] = ep->yy; c[C_EZZ][p] = ep->zz;
		c[C_EXY][p] = ep->xy; c[C_EXZ][p] = ep->xz; c[C_EYZ][p] = ep->yz;
		c[C_WXY][p] = w->xy; c[C_WXZ][p] = w->xz; c[C_WYZ][p] = w->yz;
		c[C_SXX][p] = sp->xx; c[C_SYY][p] = sp->yy; c[C_SZZ][p] = sp->zz;
		c[C_SXY][p] = sp->xy; c[C_SXZ][p] = sp->xz; c[C_SYZ][p] = sp->yz;
		c[C_P][p] = m->GetPressure();
		c[C_PXX][p] = pl->xx; c[C_PYY][p] = pl->yy; c[C_PZZ][p] = pl->zz;
		c[C_PXY][p] = pl->xy; c[C_PXZ][p] = pl->xz; c[C_PYZ][p] = pl->yz;
		const int h = historyCount[m->MatID()];
		if(h > 0) c[C_H0][p] = m->GetHistoryDble(0, 0);
		if(h > 1) c[C_H1][p] = m->GetHistoryDble(1, 0);
		c[C_WORK][p] = m->GetWorkEnergy();
		c[C_PLAST][p] = m->GetPlastEnergy();
		matCol[p] = deviceMat[m->MatID()];
		elemCol[p] = m->ElemID();
	}
	memset(&soa, 0, sizeof(soa));
	soa.n = (int64_t)n;
	soa.x = c[C_X]; soa.y = c[C_Y]; soa.z = c[C_Z];
	soa.vx = c[C_VX]; soa.vy = c[C_VY]; soa.vz = c[C_VZ];
	soa.x0 = c[C_X0]; soa.y0 = c[C_Y0]; soa.z0 = c[C_Z0];
	soa.mass = c[C_MASS];
	soa.mat = matCol.data();
	soa.elem = elemCol.data();
	soa.lpx = c[C_LPX]; soa.lpy = c[C_LPY]; soa.lpz = c[C_LPZ];
	soa.exx = c[C_EXX]; soa.eyy = c[C_EYY]; soa.ezz = c[C_EZZ];
	soa.exy = c[C_EXY]; soa.exz = c[C_EXZ]; soa.eyz = c[C_EYZ];
	soa.wxy = c[C_WXY]; soa.wxz = c[C_WXZ]; soa.wyz = c[C_WYZ];
	soa.sxx = c[C_SXX]; soa.syy = c[C_SYY]; soa.szz = c[C_SZZ];
	soa.sxy = c[C_SXY]; soa.sxz = c[C_SXZ]; soa.syz = c[C_SYZ];
	soa.pressure = c[C_P];
	soa.pxx = c[C_PXX]; soa.pyy = c[C_PYY]; soa.pzz = c[C_PZZ];
	soa.pxy = c[C_PXY]; soa.pxz = c[C_PXZ]; soa.pyz = c[C_PYZ];
	soa.hist0 = c[C_H0]; soa.hist1 = c[C_H1];
	soa.work = c[C_WORK]; soa.plast = c[C_PLAST];
}

void GPUStepTask::UnpackParticles(void)
{	const size_t n = (size_t)nmpms;
	double *c[C_COUNT];
	for(int k = 0; k < C_COUNT; k++) c[k] = cols.data() + k * n;
	for(size_t p = 0; p < n; p++)
	{	MPMBase *m = mpm[p];
		m->pos.x = c[C_X][p]; m->pos.y = c[C_Y][p];
		m->vel.x = c[C_VX][p]; m->vel.y = c[C_VY][p];
		if(dim == 3)
		{	m->pos.z = c[C_Z][p];
			m->vel.z = c[C_VZ][p];
		}
		Tensor *ep = m->GetStrainTensor(), *sp = m->GetStressTensor(), *pl = m->GetAltStrainTensor();
		TensorAntisym *w = m->GetRotationStrainTensor();
		ep->xx = c[C_EXX][p]; ep->yy = c[C_EYY][p]; ep->zz = c[C_EZZ][p];
		ep->xy = c[C_EXY][p]; ep->xz = c[C_EXZ][p]; ep->yz = c[C_EYZ][p];
		w->xy = c[C_WXY][p]; w->xz = c[C_WXZ][p]; w->yz = c[C_WYZ][p];
		sp->xx = c[C_SXX][p]; sp->yy = c[C_SYY][p]; sp->zz = c[C_SZZ][p];
		sp->xy = c[C_SXY][p]; sp->xz = c[C_SXZ][p]; sp->yz = c[C_SYZ][p];
		m->SetPressure(c[C_P][p]);
		pl->xx = c[C_PXX][p]; pl->yy = c[C_PYY][p]; pl->zz = c[C_PZZ][p];
		pl->xy = c[C_PXY][p]; pl->xz = c[C_PXZ][p]; pl->yz = c[C_PYZ][p];
		const int h = historyCount[m->MatID()];
		if(h > 0) m->SetHistoryDble(0, c[C_H0][p], 0);
		if(h > 1) m->SetHistoryDble(1, c[C_H1][p], 0);
		m->SetWorkEnergy(c[C_WORK][p]);
		// MPMBase has no setter for it: x + (-x) is exactly 0, and 0 + v is v
		m->AddPlastEnergy(-m->GetPlastEnergy());
		m->AddPlastEnergy(c[C_PLAST][p]);
		if(m->ElemID() != elemCol[p]) m->ChangeElemID(elemCol[p], false);
	}
}
