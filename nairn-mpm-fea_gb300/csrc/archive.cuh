// archive.cuh -- NairnMPM particle archive records packed on the device.
// Included by mpm_gpu.cu; implements mpmgpu_archive_record_size and
// mpmgpu_archive_records of include/nairn_mpm_gpu.h.
//
// One record per particle, in the layout of ArchiveData::ArchiveResults
// (NairnMPM/src/System/ArchiveData.cpp:807-1100) for the items of the
// MPMArchiveOrder string, after the padding and forced flags of
// ArchiveData::CalcArchiveSize (:266-283): element (int, 1-based), mass,
// material (short, 1-based, 2 pad bytes), rotation angles (3D: z, y, x degrees;
// 2D: z angle and thickness), position, original position, then the optional
// items.  Records go out in the host's particle order, so a host writes its
// 64-byte header and then this buffer.  Little-endian ('i') archives only.
#pragma once

namespace nmg {

// archive-order item indices (ArchiveData.hpp:22-32)
enum {
    ARCH_BYTE_ORDER = 0, ARCH_DEFAULTS = 1, ARCH_VELOCITY = 2, ARCH_STRESS, ARCH_STRAIN, ARCH_PLASTIC_STRAIN,
    ARCH_OLD_ORIG_POSITION, ARCH_WORK_ENERGY, ARCH_DELTA_TEMP, ARCH_PLASTIC_ENERGY, ARCH_VER2_EMPTY,
    ARCH_SHEAR_COMPONENTS, ARCH_STRAIN_ENERGY, ARCH_HISTORY, ARCH_CONCENTRATION, ARCH_HEAT_ENERGY,
    ARCH_ELEMENT_CROSSINGS, ARCH_ROT_STRAIN, ARCH_MAX_ITEMS = 25
};

// the items of one archive layout
struct ArchiveLayout {
    int dim;
    int rec;  // record bytes
    bool vel, stress, strain, plastic, work, plastE, shear, strainE, hist, conc, rot;
    double thickness;
};

// ArchiveData::CalcArchiveSize on an order string: pad with 'N', force the
// defaults, the retired items and RotStrain = Strain; refuse items the device
// does not hold (temperature, heat energy, element crossings, damage normals,
// spin, history beyond the first value, particle size) and big-endian output
inline int archive_layout(int dim, const char *order_in, ArchiveLayout &L, std::string &why) {
    if (dim != 2 && dim != 3) {
        why = "dimension must be 2 or 3";
        return MPMGPU_ERR_INVALID;
    }
    if (!order_in) {
        why = "null archive order";
        return MPMGPU_ERR_INVALID;
    }
    char o[ARCH_MAX_ITEMS + 1];
    const size_t len = std::strlen(order_in);
    for (int k = 0; k < ARCH_MAX_ITEMS; k++) o[k] = k < (int)len ? order_in[k] : 'N';
    o[ARCH_MAX_ITEMS] = 0;
    if (len < 2) {
        o[0] = 'm';
        o[1] = 'Y';
    }
    if (o[ARCH_BYTE_ORDER] != 'i') {
        why = "only little-endian ('i') archives are packed";
        return MPMGPU_ERR_UNSUPPORTED;
    }
    o[ARCH_DEFAULTS] = 'Y';
    o[ARCH_OLD_ORIG_POSITION] = 'N';
    o[ARCH_VER2_EMPTY] = 'N';
    o[ARCH_ROT_STRAIN] = o[ARCH_STRAIN];
    const int refused[] = {ARCH_DELTA_TEMP, ARCH_HEAT_ENERGY, ARCH_ELEMENT_CROSSINGS};
    for (int k : refused)
        if (o[k] != 'N') {
            why = "archive item " + std::to_string(k) + " is not held on the device";
            return MPMGPU_ERR_UNSUPPORTED;
        }
    for (int k = ARCH_ROT_STRAIN + 1; k < ARCH_MAX_ITEMS; k++)
        if (o[k] != 'N') {
            why = "archive item " + std::to_string(k) + " is not held on the device";
            return MPMGPU_ERR_UNSUPPORTED;
        }
    if (o[ARCH_HISTORY] != 'N' && o[ARCH_HISTORY] != 'Y') {
        why = "only the first history value (order 'Y') is archived from the device";
        return MPMGPU_ERR_UNSUPPORTED;
    }
    const int vec = dim == 3 ? 3 : 2, ten = dim == 3 ? 6 : 4;
    L.dim = dim;
    L.vel = o[ARCH_VELOCITY] == 'Y';
    L.stress = o[ARCH_STRESS] == 'Y';
    L.strain = o[ARCH_STRAIN] == 'Y';
    L.plastic = o[ARCH_PLASTIC_STRAIN] == 'Y';
    L.work = o[ARCH_WORK_ENERGY] == 'Y';
    L.plastE = o[ARCH_PLASTIC_ENERGY] == 'Y';
    L.shear = o[ARCH_SHEAR_COMPONENTS] == 'Y';
    L.strainE = o[ARCH_STRAIN_ENERGY] == 'Y';
    L.hist = o[ARCH_HISTORY] == 'Y';
    L.conc = o[ARCH_CONCENTRATION] == 'Y';
    L.rot = o[ARCH_ROT_STRAIN] == 'Y';
    int r = 4 + 8 + 2 + 2 + (dim == 3 ? 3 : 2) * 8 + 2 * vec * 8;
    if (L.vel) r += vec * 8;
    if (L.stress) r += ten * 8;
    if (L.strain) r += ten * 8;
    if (L.plastic) r += ten * 8;
    if (L.work) r += 8;
    if (L.plastE) r += 8;
    if (L.shear) r += 16;
    if (L.strainE) r += 8;
    if (L.hist) r += 8;
    if (L.conc) r += (1 + vec) * 8;
    if (L.rot) r += (dim == 3 ? 3 : 1) * 8;
    L.rec = r;
    return MPMGPU_OK;
}

// a double at any 4-byte aligned address (the mass follows a 4-byte int)
__device__ __forceinline__ void put_f64(char *q, double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    reinterpret_cast<unsigned *>(q)[0] = (unsigned)b;
    reinterpret_cast<unsigned *>(q)[1] = (unsigned)(b >> 32);
}

// ArchiveResults' record of slot i, written at its host index
template <int DIM>
__global__ void k_archive_pack(ArchiveLayout L, DevParticles p, const int *orig, const DevMat *mats, char *out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= p.n) return;
    char *q = out + (size_t)orig[i] * L.rec;
    int o = 0;
    auto d = [&](double v) {
        put_f64(q + o, v);
        o += 8;
    };
    const double PI = 3.14159265358979323846;
    *reinterpret_cast<int *>(q) = p.elem[i] + 1;  // ArchiveElemID, 1-based
    o = 4;
    d(p.mass[i]);
    *reinterpret_cast<short *>(q + o) = (short)(p.mat[i] + 1);  // ArchiveMatID, 1-based
    q[o + 2] = 0;
    q[o + 3] = 0;
    o += 4;
    // GetRotationZ/Y/XInDegrees with zero initial angles (MPMBase.cpp:601-622)
    d(180. * (0. - 0.5 * p.wxy[i]) / PI);
    if (DIM == 3) {
        d(180. * (0. + 0.5 * p.wxz[i]) / PI);
        d(180. * (0. - 0.5 * p.wyz[i]) / PI);
    } else {
        d(L.thickness);
    }
    d(p.x[i]);
    d(p.y[i]);
    if (DIM == 3) d(p.z[i]);
    d(p.x0[i]);
    d(p.y0[i]);
    if (DIM == 3) d(p.z0[i]);
    if (L.vel) {
        d(p.vx[i]);
        d(p.vy[i]);
        if (DIM == 3) d(p.vz[i]);
    }
    const DevMat &m = mats[p.mat[i]];
    if (L.stress) {
        // Kirchhoff stress / rho0 -> Cauchy stress: rho = rho0 / J, J the
        // relative volume (history 0 of a Neohookean material, else 1); the
        // plastic and Neohookean materials carry the pressure apart
        // (GetStressPandDev), the isotropic material does not
        const double rho = m.rho / (m.type == kMatNeohookean ? p.hist0[i] : 1.);
        const double P = m.type == kMatIsotropic ? 0. : p.pressure[i];
        d(rho * (p.sxx[i] - P));
        d(rho * (p.syy[i] - P));
        d(rho * (p.szz[i] - P));
        d(rho * p.sxy[i]);
        if (DIM == 3) {
            d(rho * p.sxz[i]);
            d(rho * p.syz[i]);
        }
    }
    if (L.strain) {
        d(p.exx[i]);
        d(p.eyy[i]);
        d(p.ezz[i]);
        d(p.exy[i]);
        if (DIM == 3) {
            d(p.exz[i]);
            d(p.eyz[i]);
        }
    }
    if (L.plastic) {
        d(p.pxx[i]);
        d(p.pyy[i]);
        d(p.pzz[i]);
        d(p.pxy[i]);
        if (DIM == 3) {
            d(p.pxz[i]);
            d(p.pyz[i]);
        }
    }
    // energies per unit mass times mass, Legacy J (UnitsController::Scaling(1.e-9))
    if (L.work) d(1.e-9 * p.mass[i] * p.work[i]);
    if (L.plastE) d(1.e-9 * p.mass[i] * p.plast[i]);
    if (L.shear) {
        // displacement gradient F - I: du/dy and dv/dx
        d(0.5 * (p.exy[i] - p.wxy[i]));
        d(0.5 * (p.exy[i] + p.wxy[i]));
    }
    if (L.strainE) d(1.e-9 * p.mass[i] * p.work[i]);  // work - residual energy (none)
    if (L.hist) d(p.hist0[i]);
    if (L.conc)
        for (int k = 0; k < (DIM == 3 ? 4 : 3); k++) d(0.);  // no transport
    if (L.rot) {
        // initial angles (GetAngle*0InDegrees): zero
        d(0.);
        if (DIM == 3) {
            d(0.);
            d(0.);
        }
    }
}

}  // namespace nmg
