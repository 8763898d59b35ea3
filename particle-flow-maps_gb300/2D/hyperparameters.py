"""Step constants of the 2D solver under the names the reference's 2D/hyperparameters.py uses
(leapfrogging vortex pairs).  Edit them here, as in the reference, before importing run_2D.  The
reference's neural-buffer and particle-reseeding constants are not used by the step and are
omitted."""
dim = 2
testing = False
save_ckpt = True
save_frame_each_step = False
use_midpoint_vel = True
use_APIC = True
forward_update_T = True
reinit_particle_pos = True

res_x = 1024
res_y = 256
visualize_dt = 0.1
reinit_every = 20
reinit_every_grad_m = 8
ckpt_every = 1
CFL = 1.0
from_frame = 0
total_frames = 5000
use_total_steps = False
total_steps = 1
exp_name = "2D_leapfrog_1024x256_reinit-20-8"

particles_per_cell = 16
total_particles_num_ratio = 1
cell_max_particle_num_ratio = 2.0
