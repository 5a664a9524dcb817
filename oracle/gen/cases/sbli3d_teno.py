"""Problem script: 3D laminar shock-wave/boundary-layer interaction, TENO5 + metrics, periodic span.

Written for this build against the reference's user API.  It is the 3D block of
apps/transitional_SBLI/transitional_SBLI.py (3D Navier-Stokes with Sutherland viscosity, metrics
stretched in x1, pressure-extrapolation inlet and extrapolation outlet in x0, isothermal wall and
shock-generator top face in x1, periodic x2, the similarity-profile initial condition,
RungeKuttaLS(3, 'SSP')) without that app's body force, statistics and restart, with the fixed TENO5
cut-off and Central(4) derivatives of the 2D benchmark case (katzer_teno.py) and the top face of the
2D case (every conserved variable piecewise constant in x0, rhou2 = 0).  The initial state is the
similarity profile with a spanwise momentum rhou2 = 0.05 sin(2 pi k / block0np2) in place of the
profile's rhou2 = 0, so that the solution varies in x2 and the x2 fluxes and derivatives are
exercised.  Grid size, dt and step count are run-time parameters.
"""
from sympy import sin, pi
from opensbli import *
from opensbli.utilities.katzer_init import Initialise_Katzer
from opensbli.utilities.helperfunctions import substitute_simulation_parameters


class SpanPerturbedKatzer(Initialise_Katzer):
    """The similarity profile of Initialise_Katzer with a periodic spanwise momentum."""

    def generate_one_wall_equations(self, *args):
        Initialise_Katzer.generate_one_wall_equations(self, *args)
        assert str(self.eqns[-1].lhs) == "rhou2"
        k = self.block.grid_indexes[2]
        self.eqns[-1] = OpenSBLIEq(DataObject('rhou2'), 0.05*sin(2*pi*k/ConstantObject('block0np2')))

ndim = 3
sc1 = "**{'scheme':'Teno'}"
mass = "Eq(Der(rho,t), - Conservative(rhou_j,x_j,%s))" % sc1
momentum = "Eq(Der(rhou_i,t) , -Conservative(rhou_i*u_j + KD(_i,_j)*p,x_j , %s) + Der(tau_i_j,x_j) )" % sc1
energy = "Eq(Der(rhoE,t), - Conservative((p+rhoE)*u_j,x_j, %s) - Der(q_j,x_j) + Der(u_i*tau_i_j ,x_j) )" % sc1
stress_tensor = "Eq(tau_i_j, (mu/Re)*(Der(u_i,x_j)+ Der(u_j,x_i) - (2/3)* KD(_i,_j)* Der(u_k,x_k)))"
heat_flux = "Eq(q_j, (-mu/((gama-1)*Minf*Minf*Pr*Re))*Der(T,x_j))"
substitutions = [stress_tensor, heat_flux]
constants = ["Re", "Pr", "gama", "Minf", "SuthT", "RefT"]
coordinate_symbol = "x"
velocity = "Eq(u_i, rhou_i/rho)"
pressure = "Eq(p, (gama-1)*(rhoE - rho*(1/2)*(KD(_i,_j)*u_i*u_j)))"
speed_of_sound = "Eq(a, (gama*p/rho)**0.5)"
temperature = "Eq(T, p*gama*Minf*Minf/(rho))"
viscosity = "Eq(mu, (T**(1.5)*(1.0+SuthT/RefT)/(T+SuthT/RefT)))"

eq = EinsteinEquation()
base_eqns = [eq.expand(e, ndim, coordinate_symbol, substitutions, constants) for e in [mass, momentum, energy]]
constituent_eqns = [eq.expand(e, ndim, coordinate_symbol, substitutions, constants)
                    for e in [velocity, pressure, speed_of_sound, temperature, viscosity]]

block = SimulationBlock(ndim, block_number=0)
metriceq = MetricsEquation()
metriceq.generate_transformations(ndim, coordinate_symbol, [(False, False), (True, False), (False, False)], 2)
simulation_eq = SimulationEquations()
constituent = ConstituentRelations()
for e in base_eqns:
    simulation_eq.add_equations(e)
for e in constituent_eqns:
    constituent.add_equations(e)
simulation_eq.apply_metrics(metriceq)

schemes = {}
teno = LLFTeno(5, averaging=RoeAverage([0, 1]))
schemes[teno.name] = teno
cent = Central(4)
schemes[cent.name] = cent
rk = RungeKuttaLS(3, formulation='SSP')
schemes[rk.name] = rk
block.set_discretisation_schemes(schemes)

local_dict = {"block": block, "GridVariable": GridVariable, "DataObject": DataObject}
x_loc = parse_expr("Eq(GridVariable(x0), block.deltas[0]*block.grid_indexes[0])", local_dict=local_dict)
boundaries = [[0, 0] for t in range(ndim)]
boundaries[0][0] = InletPressureExtrapolateBC(0, 0, scheme=ReducedAccess())
boundaries[0][1] = ExtrapolationBC(0, 1, order=0, scheme=ReducedAccess())
for con in ["Minf", "Twall"]:
    local_dict[con] = ConstantObject(con)
rhoE_wall = parse_expr("Eq(DataObject(rhoE), DataObject(rho)*Twall/(gama*(gama-1.0)*Minf**2.0))", local_dict=local_dict)
boundaries[1][0] = IsothermalWallBC(1, 0, [rhoE_wall], scheme=ReducedAccess())
top = [x_loc,
       parse_expr("Eq(DataObject(rho), Piecewise((1.129734572, (x0)>40.0), (1.00000596004, True)))", local_dict=local_dict),
       parse_expr("Eq(DataObject(rhou0), Piecewise((1.0921171, (x0)>40.0), (1.00000268202, True)))", local_dict=local_dict),
       parse_expr("Eq(DataObject(rhou1), Piecewise((-0.058866065, (x0)>40.0), (0.00565001630205, True)))", local_dict=local_dict),
       parse_expr("Eq(DataObject(rhou2), Piecewise((0.0, (x0)>40.0), (0.0, True)))", local_dict=local_dict),
       parse_expr("Eq(DataObject(rhoE), Piecewise((1.0590824, (x0)>40.0), (0.94644428042, True)))", local_dict=local_dict)]
boundaries[1][1] = DirichletBC(1, 1, top, scheme=ReducedAccess())
boundaries[2][0] = PeriodicBC(2, 0)
boundaries[2][1] = PeriodicBC(2, 1)
block.set_block_boundaries(boundaries)

for con in ["Lx1", "by"]:
    local_dict[con] = ConstantObject(con)
gridx0 = parse_expr("Eq(DataObject(x0), block.deltas[0]*block.grid_indexes[0])", local_dict=local_dict)
gridx1 = parse_expr("Eq(DataObject(x1), Lx1*sinh(by*block.deltas[1]*block.grid_indexes[1]/Lx1)/sinh(by))", local_dict=local_dict)
gridx2 = parse_expr("Eq(DataObject(x2), block.deltas[2]*block.grid_indexes[2])", local_dict=local_dict)
initial = SpanPerturbedKatzer([(False, DataObject('x0')), (True, DataObject('x1')), (False, DataObject('x2'))], 50,
                              950.0, 2.0, 288.0, [gridx0, gridx1, gridx2])

h5 = iohdf5(iotype="Write")
h5.add_arrays(simulation_eq.time_advance_arrays)
h5.add_arrays([DataObject('x0'), DataObject('x1'), DataObject('x2'), DataObject('D11')])
block.setio(h5)
block.set_equations([constituent, simulation_eq, initial, metriceq])
block.discretise()
alg = TraditionalAlgorithmRK(block)
SimulationDataType.set_datatype(Double)
OPSC(alg)
constants = ['gama', 'Minf', 'Pr', 'Re', 'Twall', 'dt', 'niter', 'block0np0', 'block0np1', 'block0np2',
             'Delta0block0', 'Delta1block0', 'Delta2block0', 'SuthT', 'RefT', 'eps', 'TENO_CT', 'Lx1', 'by']
values = ['1.4', '2.0', '0.72', '950.0', '1.67619431', '0.04', '5000', '128', '64', '16',
          '400.0/(block0np0-1)', '115.0/(block0np1-1)', '2.0', '110.4', '288.0', '1e-15', '1e-5', '115.0', '5.0']
substitute_simulation_parameters(constants, values)
