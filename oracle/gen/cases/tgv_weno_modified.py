"""Problem script: the WENO5-JS Taylor-Green vortex of tgv_weno.py with physics the GB300 kernels do not
implement, for the writer's refusal test (nothing here is run, only lowered).

OSB_PHYSICS_VARIANT selects the change: "bulk" adds a bulk-viscosity term to the stress tensor
(tau_ij gets + (1/Re) delta_ij d_k u_k), "heat" doubles the heat-flux coefficient.  The kernel names
are the same as for tgv_weno.py, so only the equations tell the difference.
"""
import os
import runpy

HERE = os.path.dirname(os.path.abspath(__file__))
variant = os.environ.get("OSB_PHYSICS_VARIANT", "bulk")
src = open(os.path.join(HERE, "tgv_weno.py")).read()
if variant == "bulk":
    old = '"Eq(tau_i_j, (1.0/Re)*(Der(u_i,x_j)+ Der(u_j,x_i)- (2/3)* KD(_i,_j)* Der(u_k,x_k)))"'
    new = '"Eq(tau_i_j, (1.0/Re)*(Der(u_i,x_j)+ Der(u_j,x_i)+ (1/3)* KD(_i,_j)* Der(u_k,x_k)))"'
else:
    old = '"Eq(q_j, (1.0/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"'
    new = '"Eq(q_j, (2.0/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"'
assert old in src
exec(compile(src.replace(old, new), os.path.join(HERE, "tgv_weno.py"), "exec"), {"__name__": "__main__"})
