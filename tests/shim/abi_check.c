/* A C99 program against include/dsrg.h, linked with libdsrg.so: every entry point the header
 * declares is taken by address (a signature that drifted from the library fails to compile or to
 * link), then one context is created.  Prints the status of dsrg_context_create (0 with a GPU). */
#include <stdio.h>

#include "dsrg.h"

typedef void (*any_function)(void);

int main(void) {
	const any_function entries[] = {
		(any_function)dsrg_context_create, (any_function)dsrg_context_destroy, (any_function)dsrg_context_last_error,
		(any_function)dsrg_context_stream, (any_function)dsrg_context_set_counting, (any_function)dsrg_context_get_stats,
		(any_function)dsrg_context_walked_fragments, (any_function)dsrg_debug_fail_allocation, (any_function)dsrg_texture_create, (any_function)dsrg_texture_create_many,
		(any_function)dsrg_texture_upload, (any_function)dsrg_texture_destroy, (any_function)dsrg_texture_read,
		(any_function)dsrg_model_create, (any_function)dsrg_model_destroy, (any_function)dsrg_model_set_bound,
		(any_function)dsrg_model_render, (any_function)dsrg_model_render_depth, (any_function)dsrg_renderer_create,
		(any_function)dsrg_renderer_destroy, (any_function)dsrg_renderer_begin, (any_function)dsrg_renderer_give_task,
		(any_function)dsrg_renderer_end, (any_function)dsrg_renderer_end_debug, (any_function)dsrg_renderer_takes_triangles,
		(any_function)dsrg_renderer_get_images, (any_function)dsrg_camera_world_to_screen, (any_function)dsrg_renderer_give_triangles,
		(any_function)dsrg_renderer_occlude_from_box, (any_function)dsrg_renderer_occlude_from_existing_triangles,
		(any_function)dsrg_renderer_occlude_from_top_rows, (any_function)dsrg_renderer_is_box_visible,
		(any_function)dsrg_renderer_has_occluders, (any_function)dsrg_renderer_get_occlusion_grid,
		(any_function)dsrg_model_render_depth_noalloc, (any_function)dsrg_batch_create, (any_function)dsrg_batch_destroy,
		(any_function)dsrg_batch_clear, (any_function)dsrg_batch_add_frame, (any_function)dsrg_batch_give_task,
		(any_function)dsrg_batch_set_depth_only, (any_function)dsrg_batch_set_tuning, (any_function)dsrg_batch_render, (any_function)dsrg_batch_autotune,
		(any_function)dsrg_context_get_tuning, (any_function)dsrg_context_set_tuning, (any_function)dsrg_diff_create,
		(any_function)dsrg_diff_destroy, (any_function)dsrg_diff_forward, (any_function)dsrg_diff_l2_loss,
		(any_function)dsrg_diff_adjoint, (any_function)dsrg_ortho_view_create, (any_function)dsrg_shadow_side_location,
		(any_function)dsrg_light_directed, (any_function)dsrg_light_points, (any_function)dsrg_light_blend,
		(any_function)dsrg_draw_higher, (any_function)dsrg_sprite_frame, (any_function)dsrg_check_float_roots, (any_function)dsrg_dense_model_create, (any_function)dsrg_dense_model_destroy,
		(any_function)dsrg_dense_render, (any_function)dsrg_dense_render_many,
	};
	size_t i, missing = 0;
	dsrg_context context = NULL;
	int status;
	for (i = 0; i < sizeof(entries) / sizeof(entries[0]); i++)
		if (!entries[i]) missing++;
	status = dsrg_context_create(0, &context);
	printf("entries %u missing %u context_create %d\n", (unsigned)(sizeof(entries) / sizeof(entries[0])), (unsigned)missing, status);
	if (context) dsrg_context_destroy(context);
	return missing == 0 ? 0 : 1;
}
