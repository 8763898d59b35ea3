"""Step constants of the 3D solver under the names the reference's 3D/hyperparameters.py uses
(case 0, two leapfrogging vortex rings).  Edit them here, as in the reference, before importing
run_3D.  The reference's neural-buffer constants are not used by the step and are omitted."""
case = 0
dim = 3

use_midpoint_vel = True
forward_update_T = True
use_APIC = True
use_APIC_smoke = True
save_particle_pos_numpy = False
save_particle_imp_numpy = False
save_frame_each_step = False
reinit_particle_pos = True

res_x = 256
res_y = 128
res_z = 128
visualize_dt = 0.1
reinit_every = 20
reinit_every_grad_m = 1
ckpt_every = 1
CFL = 0.5
from_frame = 0
total_frames = 600
use_total_steps = False
total_steps = 100
exp_name = "3D_leapfrog_reinit-20-1"

particles_per_cell = 8
total_particles_num_ratio = 1
cell_max_particle_num_ratio = 1.6
