/*
 * The atomic data source of the host tabulator: one table of function
 * pointers (xmi_atomic_data, declared in include/xmimsim_gb300.h) through
 * which every cross section and atomic parameter is read.  The default is
 * the stand-in model xrlite; a caller with xraylib and its data installs a
 * table of xraylib adapters before the first tables are built.
 */
#include <pthread.h>
#include <string.h>

#include "xmi_internal.h"
#include "xrlite.h"

static const xmi_atomic_data xrlite_table = {
    "xrlite (stand-in atomic data model)",
    xrl_AtomicWeight,
    xrl_EdgeEnergy,
    xrl_ElectronConfig,
    xrl_LineEnergy,
    xrl_RadRate,
    xrl_FluorYield,
    xrl_AugerYield,
    xrl_CosKronTransProb,
    xrl_AugerRate,
    xrl_AugerVacancies,
    xrl_CS_Total_Kissel,
    xrl_CS_Photo_Total,
    xrl_CS_Photo_Partial,
    xrl_CS_Rayl,
    xrl_CS_Compt,
    xrl_FF_Rayl,
    xrl_SF_Compt,
    xrl_DCS_Rayl,
    xrl_DCS_Compt,
    xrl_ComptonProfile,
    xrl_prepare,
};

static xmi_atomic_data installed;
static const xmi_atomic_data *current = &xrlite_table;
static pthread_mutex_t lock = PTHREAD_MUTEX_INITIALIZER;

const xmi_atomic_data *xmi_get_atomic_data(void) { return current; }

int xmi_set_atomic_data(const xmi_atomic_data *d) {
  int ok = 1;
  pthread_mutex_lock(&lock);
  if (xmi_host_tables_built()) {
    xmi_set_error("xmi_set_atomic_data: tables have been built already; install the data source first");
    ok = 0;
  } else if (!d) {
    current = &xrlite_table;
  } else if (!d->AtomicWeight || !d->EdgeEnergy || !d->ElectronConfig || !d->LineEnergy || !d->RadRate ||
             !d->FluorYield || !d->AugerYield || !d->CosKronTransProb || !d->AugerRate || !d->AugerVacancies ||
             !d->CS_Total_Kissel || !d->CS_Photo_Total || !d->CS_Photo_Partial || !d->CS_Rayl || !d->CS_Compt ||
             !d->FF_Rayl || !d->SF_Compt || !d->DCS_Rayl || !d->DCS_Compt || !d->ComptonProfile) {
    xmi_set_error("xmi_set_atomic_data: every entry but prepare must be set");
    ok = 0;
  } else {
    installed = *d;
    current = &installed;
  }
  pthread_mutex_unlock(&lock);
  return ok;
}
