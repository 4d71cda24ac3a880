/* Prints, as JSON, the size and the offset of every field of the structures that
 * cross the C ABI (include/lgx.h), as this machine's C compiler lays them out.
 * tests/test_abi_layout.py compares the Python and Rust mirrors against it. */
#include <stddef.h>
#include <stdio.h>

#include "lgx.h"

#define F(T, f) printf("%s\"%s\": [%zu, %zu]", first ? "" : ", ", #f, offsetof(T, f), \
                       sizeof(((T *)0)->f)), first = 0
#define BEGIN(name, T) printf("%s\"%s\": {\"__size__\": %zu, \"fields\": {", outer ? "" : ", ", \
                              name, sizeof(T)), outer = 0, first = 1
#define END() printf("}}")

int main(void) {
  int outer = 1, first = 1;
  printf("{");
  BEGIN("lgx_step_plan", lgx_step_plan);
  F(lgx_step_plan, mode); F(lgx_step_plan, depth); F(lgx_step_plan, words);
  F(lgx_step_plan, single_us); F(lgx_step_plan, single1_us); F(lgx_step_plan, single2_us);
  F(lgx_step_plan, wave_us); F(lgx_step_plan, temporal4_us); F(lgx_step_plan, temporal8_us);
  F(lgx_step_plan, graph_us); F(lgx_step_plan, lanes2_us); F(lgx_step_plan, lanes4_us);
  END();
  BEGIN("lgx_batch_class", lgx_batch_class);
  F(lgx_batch_class, words); F(lgx_batch_class, lattices); F(lgx_batch_class, rest);
  F(lgx_batch_class, resident); F(lgx_batch_class, cluster); F(lgx_batch_class, threads);
  F(lgx_batch_class, step_us); F(lgx_batch_class, resident_us);
  F(lgx_batch_class, steps_per_barrier); F(lgx_batch_class, word_per_thread);
  END();
  BEGIN("lgx_transport", lgx_transport);
  F(lgx_transport, nu); F(lgx_transport, g); F(lgx_transport, window_nu);
  F(lgx_transport, window_g); F(lgx_transport, u_actual); F(lgx_transport, mode_nu);
  F(lgx_transport, mode_g);
  END();
  BEGIN("lgx_request", lgx_request);
  F(lgx_request, w); F(lgx_request, h); F(lgx_request, rest_particles); F(lgx_request, seed);
  F(lgx_request, cells); F(lgx_request, density); F(lgx_request, ux); F(lgx_request, uy);
  F(lgx_request, inlet_cols); F(lgx_request, steps); F(lgx_request, sample_every);
  F(lgx_request, alpha); F(lgx_request, bx); F(lgx_request, by);
  END();
  BEGIN("lgx_server_stats", lgx_server_stats);
  F(lgx_server_stats, completed); F(lgx_server_stats, failed); F(lgx_server_stats, cancelled);
  F(lgx_server_stats, active); F(lgx_server_stats, queued); F(lgx_server_stats, ticks);
  F(lgx_server_stats, kernel_launches); F(lgx_server_stats, site_updates);
  F(lgx_server_stats, bytes_in_use); F(lgx_server_stats, peak_bytes);
  F(lgx_server_stats, peak_active); F(lgx_server_stats, gpu_busy_ns);
  F(lgx_server_stats, host_tick_ns); F(lgx_server_stats, host_wait_ns);
  END();
  printf("}\n");
  return 0;
}
