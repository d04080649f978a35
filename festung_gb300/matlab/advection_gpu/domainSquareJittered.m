% core/domainSquare.m on [0,1]^2 with its interior nodes moved by uniform noise of +-jitter*h in
% each coordinate (seeded), then the grid data rebuilt (core/generateGridData.m) and the boundary
% ids set as core/domainSquare.m:97-104 does.  jitter = 0 is domainSquare itself.
function g = domainSquareJittered(hmax, jitter, seed)
g = domainSquare(hmax);
if jitter <= 0
  return
end % if
h = 1 / ceil(1 / hmax);
s = RandStream('mt19937ar', 'Seed', seed);
d = (2 * rand(s, g.numV, 2) - 1) * (jitter * h);
coordV = g.coordV;
interior = coordV(:,1) > 0 & coordV(:,1) < 1 & coordV(:,2) > 0 & coordV(:,2) < 1;
coordV(interior, :) = coordV(interior, :) + d(interior, :);
g = generateGridData(coordV, g.V0T);
g.idE = zeros(g.numE, 1);
tol = 10*eps;
g.idE(abs(g.baryE(:, 2)) < tol) = 1;       % south
g.idE(abs(g.baryE(:, 1) - 1) < tol) = 2;   % east
g.idE(abs(g.baryE(:, 2) - 1) < tol) = 3;   % north
g.idE(abs(g.baryE(:, 1)) < tol) = 4;       % west
g.idE0T = g.idE(g.E0T);
end % function
