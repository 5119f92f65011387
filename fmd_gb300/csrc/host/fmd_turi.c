/* placeholder: continuum grids are added in the TTM milestone */
#include <stdlib.h>
#include "fmd_private.h"

void _fmdh_turies_free(fmd_t *md) { (void)md; }
void _fmdh_turies_update(fmd_t *md, bool xupd, bool vupd, bool fupd) { (void)md; (void)xupd; (void)vupd; (void)fupd; }
void _fmdh_ttm_get_ready(fmd_t *md) { (void)md; }
void _fmdh_se_integrate(fmd_t *md, double duration) { (void)md; (void)duration; }

fmd_handle_t fmd_turi_add(fmd_t *md, fmd_turi_t cat, int dimx, int dimy, int dimz, fmd_real_t starttime, fmd_real_t stoptime)
{ (void)cat; (void)dimx; (void)dimy; (void)dimz; (void)starttime; (void)stoptime;
  FMD_ERR(md, FMD_ERR_NOT_SUPPORTED_YET, false, "turi"); return -1; }
fmd_handle_t fmd_field_find(fmd_t *md, fmd_handle_t turi, fmd_field_t cat) { (void)md; (void)turi; (void)cat; return -1; }
fmd_handle_t fmd_field_add(fmd_t *md, fmd_handle_t turi, fmd_field_t cat, fmd_real_t interval) { (void)md; (void)turi; (void)cat; (void)interval; return -1; }
void fmd_field_save_as_hdf5(fmd_t *md, fmd_handle_t turi, fmd_handle_t field, fmd_string_t filename) { (void)md; (void)turi; (void)field; (void)filename; }
fmd_array3s_t *fmd_field_getArray(fmd_t *md, fmd_handle_t turi, fmd_handle_t field, fmd_array3_t *array, fmd_utriple_t dims) { (void)md; (void)turi; (void)field; (void)array; (void)dims; return NULL; }
void fmd_array3s_free(fmd_array3s_t *array) { (void)array; }
void _fmd_ttm_setHeatCapacity_linear(fmd_t *md, fmd_handle_t turi, fmd_ttm_heat_capacity_linear_t c) { (void)md; (void)turi; (void)c; }
void _fmd_ttm_setHeatCapacity_file(fmd_t *md, fmd_handle_t turi, fmd_string_t path) { (void)md; (void)turi; (void)path; }
void _fmd_ttm_setHeatConductivity_constant1(fmd_t *md, fmd_handle_t turi, fmd_real_t k) { (void)md; (void)turi; (void)k; }
void _fmd_ttm_setHeatConductivity_constant2(fmd_t *md, fmd_handle_t turi, fmd_ttm_heat_conductivity_constant_t k) { (void)md; (void)turi; (void)k; }
void _fmd_ttm_setHeatConductivity_zhigilei(fmd_t *md, fmd_handle_t turi, fmd_ttm_heat_conductivity_zhigilei_t k) { (void)md; (void)turi; (void)k; }
void _fmd_ttm_setCouplingFactor_constant1(fmd_t *md, fmd_handle_t turi, fmd_real_t g) { (void)md; (void)turi; (void)g; }
void _fmd_ttm_setCouplingFactor_constant2(fmd_t *md, fmd_handle_t turi, fmd_ttm_coupling_factor_constant_t g) { (void)md; (void)turi; (void)g; }
void _fmd_ttm_setCouplingFactor_file(fmd_t *md, fmd_handle_t turi, fmd_string_t path) { (void)md; (void)turi; (void)path; }
void fmd_ttm_setElectronTemperature(fmd_t *md, fmd_handle_t turi, fmd_real_t Te) { (void)md; (void)turi; (void)Te; }
void fmd_ttm_setTimestepRatio(fmd_t *md, fmd_handle_t turi, int ratio) { (void)md; (void)turi; (void)ratio; }
void fmd_ttm_setCellActivationFraction(fmd_t *md, fmd_handle_t turi, fmd_real_t value) { (void)md; (void)turi; (void)value; }
void _fmd_ttm_setLaserSource_gaussian(fmd_t *md, fmd_handle_t turi, fmd_ttm_laser_gaussian_t laser) { (void)md; (void)turi; (void)laser; }
