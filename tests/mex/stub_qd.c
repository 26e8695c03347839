/*
 * stub_qd.c - stand-in for libqd's qd_evolve, for CPU tests of the MEX shim.
 *
 * TEST INFRASTRUCTURE.  Follows libqd's host-side contract without a GPU: one
 * "step" writes the number of steps done into wave_packets[0]; the callback
 * fires after the step whose counter (before the increment) is a multiple of
 * steps_to_copy_psi_from_device_to_host, with time.steps holding that counter;
 * a non-zero callback return ends the run with QD_ERR_CALLBACK; time.steps
 * holds the steps done on return.  stub_live_sessions() counts runs whose
 * clean-up (the library's session destructor) has not run: non-zero after a
 * MEX error would mean the shim unwound through the library.
 */
#include <stdio.h>

#include "qd.h"

static int g_live = 0;
static char g_err[128] = "";

int stub_live_sessions(void) { return g_live; }

int qd_evolve(qd_fh2data *d, qd_callback cb, void *user) {
  g_live++;
  g_err[0] = '\0';
  int status = QD_OK;
  const int every = d->options.wave_to_matlab ? d->options.steps_to_copy_psi_from_device_to_host : 0;
  for (int k = 0; k < d->time.total_steps; k++) {
    const int counter = d->time.steps;
    d->OmegaStates.wave_packets[0] = counter + 1.0;
    if (cb && every > 0 && counter % every == 0) {
      d->time.steps = counter;
      if (cb(d, user) != 0) {
        d->time.steps = counter + 1;
        status = QD_ERR_CALLBACK;
        snprintf(g_err, sizeof g_err, "wave_to_matlab callback returned an error");
        break;
      }
    }
    d->time.steps = counter + 1;
  }
  g_live--;   /* the session's destructor */
  return status;
}

const char *qd_last_error(void) { return g_err; }
int qd_version(void) { return QD_VERSION; }
